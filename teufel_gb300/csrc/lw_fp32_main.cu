// lw_fp32_main.cu -- the split-precision field integration: per-point
// preparation, the per-pixel-range kernel, the kernel dispatch, and the
// diagnostics that run the same device functions (lw_fp32_point.cuh).
//
// One thread owns one observation point (pixel); a 2-D grid spans pixel
// blocks x particle-range slots.  For every particle of its slot a thread
// bisects the particle's trajectory for the steps whose arrival overlaps its
// trace window, then walks those steps, evaluating each trajectory point
// once (the reference evaluates it twice, src/particle.cpp:788-798) and
// depositing each step with the interval-overlap weighting of
// ChargedParticle::integrateFieldTrace (src/particle.cpp:771-867).  The
// warp-uniform kernel (lw_fp32_warp.cu) walks the union of a warp's ranges
// with the trajectory staged in shared memory.
//
// Arrival times.  Every kSegLen steps an FP64 "anchor" gives the arrival time
// of the segment's first point, through the exact far-field identity
//    |P - x| = L + G,  L = |P| - P^.x,  G = |x x P^|^2 / (L + |P - x|)
//    ts - t0 = (|P|/c - t0) + (t - P^.x/c) + G/c
// where |P|/c - t0 is formed once per pixel in double-float arithmetic, so no
// term of the size of the flight time P/c is ever rounded.  Between anchors
// the arrival time advances step by step by the exact increment
//    ts(i+1) - ts(i) = dt_i (1 - beta_c . n_m),
//    beta_c = (x(i+1)-x(i))/(c dt_i),  n_m = (D_i + D_(i+1))/(R_i + R_(i+1))
// evaluated in FP32 in split form (chord 1-|beta_c| precomputed in FP64) and
// summed with compensation.  A point's arrival is held as an integer bin plus
// an FP32 remainder in [-1/2, 1/2], so weights never lose bits to offsets.
//
// Bin indices and window decisions are bit-identical to the reference: when
// the estimate lies within its error bound (the reference's own rounding plus
// ours) of a half-integer, the point is re-evaluated with the reference's
// exact FP64 operation sequence (exact_retarded_time).
//
// Field (FP32), with W = beta_hat x N, c1 = 1 + beta_hat.N:
//    kappa = 1 - n.beta = eps + |beta| |W|^2 / c1,            eps = 1 - |beta|
//    N - beta = W x (N + beta_hat) / c1 + beta_hat * eps
//    E = (N-beta) scale/(gamma^2 R^2 kappa^3) + N x ((N-beta) x beta') scale/(c R kappa^3)
//    B c = N x E   (1/c applied in the FP64 reduction)
#include <cuda_runtime.h>

#include "lw_fp32_point.cuh"

namespace teufel {

// ---------------------------------------------------------------------------
// Per-point preparation (pixel independent), run once after upload
// ---------------------------------------------------------------------------
// One warp per particle: the lanes test the steps in parallel.  vhat.w is
// the particle's smallest arrival advance of a step, min(dt - |dx|/c) > 0:
// every observer's arrival time then grows by at least that much per step
// (triangle inequality), which the range bisection relies on.  It is 0 when
// some step does not run forward in time or is not slower than light, and
// 1e300 for a particle without steps.
__global__ void prep_particles_kernel(DevTraj tr, double4_32a* vhat) {
    const int m = blockIdx.x;
    if (m >= tr.n_particles) return;
    const int64_t o = tr.offsets[m], n = tr.offsets[m + 1] - o;
    double min_inc = 1e300;
    for (int64_t i = o + threadIdx.x; i + 1 < o + n; i += 32) {
        const double4_32a p = tr.tx[i], q = tr.tx[i + 1];
        const double ddt = q.x - p.x;
        const double ex = q.y - p.y, ey = q.z - p.z, ez = q.w - p.w;
        const double inc = ddt - sqrt(ex * ex + ey * ey + ez * ez) / kC;
        min_inc = (ddt > 0.0 && inc > 0.0) ? fmin(min_inc, inc) : 0.0;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) min_inc = fmin(min_inc, __shfl_xor_sync(0xffffffffu, min_inc, d));
    if (threadIdx.x != 0) return;
    double4_32a v = make_double4_32a(0.0, 0.0, 1.0, 1e300);
    if (n >= 2) {
        const double4_32a a = tr.tx[o], b = tr.tx[o + n - 1];
        const double dx = b.y - a.y, dy = b.z - a.z, dz = b.w - a.w;
        const double L = sqrt(dx * dx + dy * dy + dz * dz);
        if (L > 0.0) v = make_double4_32a(dx / L, dy / L, dz / L, 0.0);
        v.w = min_inc;
    }
    vhat[m] = v;
}

cudaError_t launch_prep_particles(const DevTraj& tr, cudaStream_t s) {
    if (tr.n_particles > 0)
        prep_particles_kernel<<<tr.n_particles, 32, 0, s>>>(tr, const_cast<double4_32a*>(tr.vhat));
    return cudaGetLastError();
}

__global__ void prep_points_kernel(DevTraj tr, float4* q0, float4* q1, float4* q2, float4* q3) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tr.n_points) return;
    int lo = 0, hi = tr.n_particles - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tr.offsets[mid] <= i) lo = mid; else hi = mid - 1;
    }
    const int m = lo;
    const int64_t o = tr.offsets[m], n = tr.offsets[m + 1] - o;
    const int64_t ia = o + ((i - o) & ~(int64_t)(kSegLen - 1));
    double4_32a p = tr.tx[i], a = tr.tx[ia];
    // chord of the step i -> i+1
    double ddt = 0.0, cx = 0.0, cy = 0.0, cz = 1.0, ceps = 1.0;
    if (i + 1 < o + n) {
        double4_32a q = tr.tx[i + 1];
        ddt = q.x - p.x;
        double ex = q.y - p.y, ey = q.z - p.z, ez = q.w - p.w;
        double L = sqrt(ex * ex + ey * ey + ez * ez);
        if (L > 0.0) {
            cx = ex / L;
            cy = ey / L;
            cz = ez / L;
        }
        double cd = kC * ddt;
        ceps = cd != 0.0 ? (cd - L) / cd : 1.0;  // 1 - |chord velocity|/c
    }
    double ex = p.y - a.y, ey = p.z - a.z, ez = p.w - a.w;
    to_frame(tr.frame, ex, ey, ez);
    to_frame(tr.frame, cx, cy, cz);
    q0[i] = make_float4((float)ex, (float)ey, (float)ez, (float)ddt);
    q3[i] = make_float4((float)cx, (float)cy, (float)cz, (float)ceps);
    double4_32a bg = tr.pp[i], ac = tr.aa[i];
    double P = sqrt(bg.x * bg.x + bg.y * bg.y + bg.z * bg.z);
    double gamma = sqrt(P * P + 1.0);
    double bx = 0.0, by = 0.0, bz = 1.0, eps = 1.0;
    if (P > 0.0) {
        bx = bg.x / P;
        by = bg.y / P;
        bz = bg.z / P;
        eps = 1.0 / (gamma * (gamma + P));  // 1 - |beta| without cancellation
    }
    to_frame(tr.frame, bx, by, bz);
    q1[i] = make_float4((float)bx, (float)by, (float)bz, (float)eps);
    double scale = field_scale(tr.charge[m]);
    double sa = scale / (gamma * kC);
    double ax = ac.x, ay = ac.y, az = ac.z;
    to_frame(tr.frame, ax, ay, az);
    q2[i] = make_float4((float)(ax * sa), (float)(ay * sa), (float)(az * sa),
                        (float)(scale / (gamma * gamma)));
}

// After the set's frame is known (from the particles' directions).
cudaError_t launch_prep_points(const DevTraj& tr, cudaStream_t s) {
    if (tr.n_points > 0) {
        unsigned blocks = (unsigned)((tr.n_points + 255) / 256);
        prep_points_kernel<<<blocks, 256, 0, s>>>(tr, const_cast<float4*>(tr.q0),
                                                  const_cast<float4*>(tr.q1),
                                                  const_cast<float4*>(tr.q2),
                                                  const_cast<float4*>(tr.q3));
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Kernel 2 (lane-divergent): every pixel walks its own in-window steps, its
// start aligned to a segment boundary so that a warp changes anchors
// together; trajectory data is read per lane from global memory.  Best when
// neighbouring pixels see a particle at very different times.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128, 4)
    lw_fp32_lanes_kernel(DevTraj tr, DevScreen sc, DevWork wk) {
    __shared__ PixelCtx pxs[128];
    const int slot = blockIdx.y;
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = pix < sc.np;
    const int pc = active ? pix : sc.np - 1;
    const double3 P = make_double3(sc.pix_pos[3 * pc], sc.pix_pos[3 * pc + 1],
                                   sc.pix_pos[3 * pc + 2]);
    pxs[threadIdx.x] = make_pixel(P, sc.pix_t0[pc], sc.dt, sc.nt);
    const PixelCtx& px = pxs[threadIdx.x];
    PrefetchSink sink;
    sink.init(static_cast<float*>(wk.scratch) + (int64_t)slot * wk.slot_stride +
                  (int64_t)pc * sc.nt * 6,
              sc.nt);
    const int64_t g0 = wk.slot_seg[slot], g1 = wk.slot_seg[slot + 1];
    int m = g0 < g1 ? particle_of_segment(tr.seg_offsets, tr.n_particles, g0) : tr.n_particles;
    unsigned long long inwin = 0, nfb = 0, nev = 0;
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
        if (!active) last = first - 1;
        int start = first & ~(kSegLen - 1);
        if (start < st_lo) start = st_lo;
        const int trips = last >= first ? last - start + 1 : 0;
        const int max_trips = warp_max(trips);
        if (max_trips == 0) continue;
        if (trips == 0) start = st_lo;
        else nev += (unsigned long long)(trips + 1);
        const double4_32a* txp = tr.tx + po;
        const float4 *q0 = tr.q0 + po, *q1 = tr.q1 + po, *q2 = tr.q2 + po, *q3 = tr.q3 + po;
        Anchor A;
        make_anchor(A, txp[start], px, tr.frame);
        PointState p1, p2;
        point_field(p1, __ldg(q0 + start), __ldg(q1 + start), __ldg(q2 + start), A);
        start_chain(p1, A);
        if (decide(p1, A.err, txp, start, px, A)) nfb++;
        float comp = 0.0f, chain_err = 0.0f;
        for (int j = 0; j < max_trips; ++j) {
            const int i2 = start + j + 1;
            const bool live = j < trips;
            // uniform: every lane's start is a segment boundary, so the lanes
            // reach segment and chunk boundaries together
            const bool boundary = (i2 & (kSegLen - 1)) == 0 ||
                                  ((i2 & (kChunkLen - 1)) == 0 &&
                                   warp_any_above(chain_err, kReanchorBound));
            if (boundary) {
                const int i2c = i2 < npm ? i2 : ((npm - 1) & ~(kChunkLen - 1));
                Anchor An;
                make_anchor(An, txp[i2c], txp[i2c & ~(kSegLen - 1)], px, tr.frame);
                rebase(p1, A, An);
                A = An;
            }
            if (live) {
                point_field(p2, __ldg(q0 + i2), __ldg(q1 + i2), __ldg(q2 + i2), A);
                if (boundary) {
                    start_chain(p2, A);
                    comp = 0.0f;
                    chain_err = 0.0f;
                } else {
                    const float du = step_increment(p1, p2, __ldg(q3 + i2 - 1), px.kdt);
                    chain_step(p1, p2, du, comp);
                    chain_err += fabsf(du) * kChainRel + 1.0e-7f;
                }
                if (decide(p2, A.err + chain_err, txp, i2, px, A)) nfb++;
                if (deposit_step32(p1, p2, A.Bi, sc.nt, sink)) inwin++;
                p1 = p2;
            }
        }
    }
    sink.flush();
    if (sink.err) atomicOr(wk.status, sink.err);
    inwin = warp_sum_u64(inwin);
    nfb = warp_sum_u64(nfb);
    unsigned long long nadd = warp_sum_u64(sink.n_add);
    nev = warp_sum_u64(nev);
    if ((threadIdx.x & 31) == 0 && wk.counters) {
        if (inwin) atomicAdd(wk.counters, inwin);
        if (nfb) atomicAdd(wk.counters + 1, nfb);
        if (nadd) atomicAdd(wk.counters + 2, nadd);
        if (nev) atomicAdd(wk.counters + 3, nev);
    }
}

cudaError_t launch_fp32(const DevTraj& tr, const DevScreen& sc, const DevWork& w, int variant,
                        cudaStream_t s) {
    if (variant == kVariantLanes) {
        dim3 grid((sc.np + 127) / 128, w.n_slots);
        lw_fp32_lanes_kernel<<<grid, 128, 0, s>>>(tr, sc, w);
        return cudaGetLastError();
    }
    if (is_pair_variant(variant)) return launch_fp32_pair(tr, sc, w, variant, s);
    return launch_fp32_warp(tr, sc, w, variant, s);
}

// ---------------------------------------------------------------------------
// Injected arrival times and fields through the FP32 deposit above (the
// reference's known-answer test injects them by overriding
// RetardedTime/RetardedField, tests/teufel.integrate_field.cpp:51-78).
// One thread; particles in order; partial trace in FP32 then added to trace.
// ---------------------------------------------------------------------------
__global__ void deposit_injected32_kernel(int n_part, const int64_t* offs, const double* ts,
                                          const double* f, double t0, double dt, int nt,
                                          double* trace, float* trace32, unsigned int* status) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const Window w = make_window(t0, dt, nt);
    PrefetchSink sink;
    sink.init(trace32, nt);
    for (int m = 0; m < n_part; m++) {
        const int64_t o = offs[m], n = offs[m + 1] - o;
        PointState p1, p2;
        for (int64_t s = 0; s < n; s++) {
            const double t = ts[o + s];
            double u = (t - t0) / dt;
            u = fmax(-kBinLimit, fmin(u, kBinLimit));
            const double k = floor(u + 0.5);
            p2.ki = (int)k;
            p2.r = (float)(u - k);
            p2.idx = exact_bin(t, w);
            p2.flags = exact_flags(t, w);
            for (int c = 0; c < 3; c++)
                p2.f[c] = make_float2((float)f[6 * (o + s) + 2 * c], (float)f[6 * (o + s) + 2 * c + 1]);
            if (s > 0) deposit_step32(p1, p2, 0, nt, sink);
            p1 = p2;
        }
    }
    sink.flush();
    for (int k = 0; k < 6 * nt; k++) trace[k] += (double)trace32[k];
    if (sink.err) atomicOr(status, sink.err);
}

cudaError_t launch_deposit_injected32(int n_part, const int64_t* offs, const double* ts,
                                      const double* f, double t0, double dt, int nt,
                                      double* trace, float* trace32, unsigned int* status,
                                      cudaStream_t s) {
    deposit_injected32_kernel<<<1, 32, 0, s>>>(n_part, offs, ts, f, t0, dt, nt, trace, trace32,
                                               status);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Decision record for the parity tests: one thread per segment of particle
// m walks its points as both kernels do (anchor, FP32 chain, decision), with
// the longest chain they can run (a whole segment, no intermediate anchor),
// so that the error bound is checked where it is widest.  u_est is the
// estimate before any exact fallback, band the bound used.
// ---------------------------------------------------------------------------
__global__ void point_decisions_kernel(DevTraj tr, int m, double3 P, double t0, double dt,
                                       int nt, int64_t* idx, int* flags, double* u_est,
                                       float* band) {
    const int64_t o = tr.offsets[m];
    const int n = (int)(tr.offsets[m + 1] - o);
    const int seg = blockIdx.x * blockDim.x + threadIdx.x;
    const int start = seg << kSegShift;
    if (start >= n) return;
    const PixelCtx px = make_pixel(P, t0, dt, nt);
    const double4_32a* txp = tr.tx + o;
    Anchor A;
    make_anchor(A, txp[start], px, tr.frame);
    PointState p1, p2;
    float comp = 0.0f, chain_err = 0.0f;
    for (int i = start; i < n && i < start + kSegLen; i++) {
        point_field(p2, tr.q0[o + i], tr.q1[o + i], tr.q2[o + i], A);
        if (i == start) {
            start_chain(p2, A);
        } else {
            const float du = step_increment(p1, p2, tr.q3[o + i - 1], px.kdt);
            chain_step(p1, p2, du, comp);
            chain_err += fabsf(du) * kChainRel + 1.0e-7f;
        }
        u_est[i] = (double)A.B + (double)p2.ki + (double)p2.r;
        if (band) band[i] = A.err + chain_err;
        decide(p2, A.err + chain_err, txp, i, px, A);
        idx[i] = p2.idx;
        flags[i] = p2.flags;
        p1 = p2;
    }
}

cudaError_t launch_point_decisions(const DevTraj& tr, int m, double3 pos, double t0, double dt,
                                   int nt, int64_t n_points, int64_t* idx, int* flags,
                                   double* u_est, float* band, cudaStream_t s) {
    if (n_points <= 0) return cudaSuccess;
    const int64_t nseg = (n_points + kSegLen - 1) / kSegLen;
    point_decisions_kernel<<<(unsigned)((nseg + 127) / 128), 128, 0, s>>>(tr, m, pos, t0, dt, nt,
                                                                         idx, flags, u_est, band);
    return cudaGetLastError();
}

}  // namespace teufel
