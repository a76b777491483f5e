// lw_fp32_warp.cu -- the warp-uniform split-precision kernel (the default).
//
// Each warp owns 32 pixels and works on its own: for every particle of its
// slot it walks the union of its lanes' in-window step ranges, all 32 lanes on
// the same trajectory point at the same time.  The particle's per-point data
// (64 B per point) is staged into the warp's own shared-memory double buffer,
// one chunk (kChunkLen points) at a time, with cp.async; every lane then reads
// it as a broadcast.  The arrival chain starts at the first chunk of the walk
// and is re-anchored in FP64 at every segment boundary (every kSegLen points)
// and at any chunk boundary where its error bound has grown past
// kReanchorBound.  No block-wide barrier is involved, so warps never wait
// for one another, and a warp's step range is only as wide as its own 32
// pixels need.  The per-point work is in lw_fp32_point.cuh.
#include <cuda_runtime.h>

#include "lw_fp32_point.cuh"

namespace teufel {

constexpr int kWThreads = 256;
constexpr int kWWarps = kWThreads / 32;

struct __align__(16) WarpChunk {
    float4 q0[kChunkLen], q1[kChunkLen], q2[kChunkLen], q3[kChunkLen];
};

// The 32 lanes copy the four per-point arrays of `avail` points starting at p0.
__device__ __forceinline__ void warp_stage(WarpChunk* b, const DevTraj& tr, int64_t p0, int avail,
                                           int lane) {
#pragma unroll
    for (int k = 0; k < 4 * kChunkLen / 32; k++) {
        const int t = lane + 32 * k;
        const int arr = t / kChunkLen, l = t % kChunkLen;
        if (l < avail) {
            const float4* src = arr == 0 ? tr.q0 : arr == 1 ? tr.q1 : arr == 2 ? tr.q2 : tr.q3;
            float4* dst = arr == 0 ? b->q0 : arr == 1 ? b->q1 : arr == 2 ? b->q2 : b->q3;
            const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + l);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa),
                         "l"(src + p0 + l)
                         : "memory");
        }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// MINB = resident blocks per SM the register allocation is sized for.
template <int MINB>
__global__ void __launch_bounds__(kWThreads, MINB)
    lw_fp32_warp_kernel(DevTraj tr, DevScreen sc, DevWork wk) {
    __shared__ WarpChunk buf[kWWarps][2];
    // the FP64 pixel constants are needed only at anchors and in the exact
    // fallback: kept in shared memory rather than in registers
    __shared__ PixelCtx pxs[kWThreads];
    const int slot = blockIdx.y;
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool active = pix < sc.np;
    const int pc = active ? pix : sc.np - 1;
    const double3 P = make_double3(sc.pix_pos[3 * pc], sc.pix_pos[3 * pc + 1],
                                   sc.pix_pos[3 * pc + 2]);
    pxs[threadIdx.x] = make_pixel(P, sc.pix_t0[pc], sc.dt, sc.nt);
    const PixelCtx& px = pxs[threadIdx.x];
    WarpChunk* wb = buf[warp];
    RedSink sink;
    sink.init(static_cast<float*>(wk.scratch) + (int64_t)slot * wk.slot_stride +
                  (int64_t)pc * sc.nt * 6,
              sc.nt);
    const int64_t g0 = wk.slot_seg[slot], g1 = wk.slot_seg[slot + 1];
    int m = g0 < g1 ? particle_of_segment(tr.seg_offsets, tr.n_particles, g0) : tr.n_particles;
    unsigned long long inwin = 0, nfb = 0, nev = 0;
    float4 q3_last = make_float4(0.0f, 0.0f, 1.0f, 1.0f);  // chord of a chunk's last step
    for (; m < tr.n_particles && tr.seg_offsets[m] < g1; ++m) {
        const int64_t sb = tr.seg_offsets[m];
        const int64_t po = tr.offsets[m];
        const int npm = (int)(tr.offsets[m + 1] - po);
        const int lg0 = (int)((g0 > sb ? g0 : sb) - sb);
        const int64_t se = tr.seg_offsets[m + 1];
        const int lg1 = (int)((g1 < se ? g1 : se) - sb);
        const int st_lo = lg0 << kSegShift;
        int st_hi = lg1 << kSegShift;
        if (st_hi > npm - 1) st_hi = npm - 1;
        if (st_lo >= st_hi) continue;  // uniform over the block
        int first = st_lo, last = st_hi - 1;
        if (tr.vhat[m].w > 0.0)
            inwindow_steps(tr.tx + po, st_lo, st_hi, P, px.w, tr.vhat[m].w, &first, &last);
        if (!active || last < first) {
            first = 0x7fffffff;
            last = -1;
        }
        const int lo = warp_min(first), hi = warp_max(last);
        if (lo > hi) continue;  // uniform over the warp
        const int start = lo & ~(kChunkLen - 1);  // >= st_lo, a segment boundary
        const int n_pts = hi + 2 - start;           // points start .. hi+1
        const int n_chunks = (n_pts + kChunkLen - 1) >> kChunkShift;
        const double4_32a* txp = tr.tx + po;
        warp_stage(&wb[0], tr, po + start, min(kChunkLen, npm - start), lane);
        Anchor A;
        PointState p1, p2;
        float comp = 0.0f, chain_err = 0.0f;
        bool reg1 = false;
        for (int c = 0; c < n_chunks; c++) {
            const int p0 = start + (c << kChunkShift);
            if (c + 1 < n_chunks) {
                warp_stage(&wb[(c + 1) & 1], tr, po + p0 + kChunkLen,
                           min(kChunkLen, npm - (p0 + kChunkLen)), lane);
                asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            } else {
                asm volatile("cp.async.wait_group 0;\n" ::: "memory");
            }
            __syncwarp();
            const WarpChunk& B = wb[c & 1];
            // a new chain at the start of the walk, at every segment boundary,
            // and where the error bound of a lane has grown too large
            const bool anchor = c == 0 || (p0 & (kSegLen - 1)) == 0 ||
                                warp_any_above(chain_err, kReanchorBound);
            if (anchor) {
                Anchor An;
                make_anchor(An, txp[p0], txp[p0 & ~(kSegLen - 1)], px, tr.frame);
                if (c > 0) rebase(p1, A, An);
                A = An;
            }
            const int n_here = min(kChunkLen, n_pts - (c << kChunkShift));
            for (int l = 0; l < n_here; l++) {
                const int i = p0 + l;
                point_field(p2, B.q0[l], B.q1[l], B.q2[l], A);
                if (l == 0 && anchor) {
                    start_chain(p2, A);
                    comp = 0.0f;
                    chain_err = 0.0f;
                } else {
                    const float du = step_increment(p1, p2, l > 0 ? B.q3[l - 1] : q3_last, px.kdt);
                    chain_step(p1, p2, du, comp);
                    chain_err += fabsf(du) * kChainRel + 1.0e-7f;
                }
                bool reg2;
                if (0.5f - fabsf(p2.r) <= A.err + chain_err) {
                    apply_exact(p2, exact_point(txp, i, px, A.Bi));
                    nfb++;
                    reg2 = false;
                } else {
                    p2.flags = 0;
                    reg2 = (unsigned)(A.Bi + p2.ki) < (unsigned)sc.nt;
                }
                const bool dep = i > start && active;
                const bool fast = reg1 && reg2 && (unsigned)(p2.ki - p1.ki) <= 1u;
                if (__all_sync(0xffffffffu, fast || !dep)) {
                    if (dep) {
                        deposit_fast(p1, p2, A.Bi, sink);
                        inwin++;
                    }
                } else if (dep) {
                    materialize(p1, A.Bi, sc.nt);
                    materialize(p2, A.Bi, sc.nt);
                    if (deposit_step32(p1, p2, A.Bi, sc.nt, sink)) inwin++;
                }
                reg1 = reg2;
                p1 = p2;
            }
            q3_last = B.q3[kChunkLen - 1];
            __syncwarp();  // the buffer is restaged two chunks later
        }
        if (active) nev += (unsigned long long)n_pts;
    }
    sink.flush();
    if (sink.err) atomicOr(wk.status, sink.err);
    inwin = warp_sum_u64(active ? inwin : 0);
    nfb = warp_sum_u64(active ? nfb : 0);
    unsigned long long nadd = warp_sum_u64(sink.n_add);
    nev = warp_sum_u64(nev);
    if (lane == 0 && wk.counters) {
        if (inwin) atomicAdd(wk.counters, inwin);
        if (nfb) atomicAdd(wk.counters + 1, nfb);
        if (nadd) atomicAdd(wk.counters + 2, nadd);
        if (nev) atomicAdd(wk.counters + 3, nev);
    }
}

cudaError_t launch_fp32_warp(const DevTraj& tr, const DevScreen& sc, const DevWork& w,
                             int variant, cudaStream_t s) {
    dim3 grid((sc.np + kWThreads - 1) / kWThreads, w.n_slots);
    if (variant == kVariantWarp3)
        lw_fp32_warp_kernel<3><<<grid, kWThreads, 0, s>>>(tr, sc, w);
    else
        lw_fp32_warp_kernel<2><<<grid, kWThreads, 0, s>>>(tr, sc, w);
    return cudaGetLastError();
}

}  // namespace teufel
