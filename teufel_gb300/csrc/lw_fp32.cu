// lw_fp32.cu -- the split-precision field-integration kernel.
//
// One thread owns one observation point (pixel); a 2-D grid spans pixel
// blocks x particle-range slots.  For every particle of its slot a thread
// bisects the particle's trajectory for the steps whose arrival overlaps its
// trace window, then walks those steps, evaluating each trajectory point
// once (the reference evaluates it twice, src/particle.cpp:788-798) and
// depositing each step with the interval-overlap weighting of
// ChargedParticle::integrateFieldTrace (src/particle.cpp:771-867).
//
// Precision split:
//  * FP64 only per segment of kSegLen steps ("anchor"): distance, direction
//    and arrival time of the segment's first point, plus the exact fallback.
//  * FP32 per point: the arrival time relative to the anchor through
//    cancellation-free forms, and the Lienard-Wiechert field
//    (src/particle.cpp:570-596) with 1 - n.beta in split form.
//  * Bin indices and window decisions are bit-identical to the reference:
//    when the FP32 estimate of (ts-t0)/dt lies within its error bound of a
//    half-integer, the point is re-evaluated with the reference's exact FP64
//    arithmetic (exact_retarded_time).
//
// Arrival time relative to the anchor a (exact identities, D_a = P - x_a,
// R_a = |D_a|, n_a = D_a/R_a, e = x - x_a, v = the particle's frame direction):
//    R   = R_a - n_a.e + |e x n_a|^2 / (R + R_a - n_a.e)
//    ts - ts_a = [(t - t_a) - v.e/c] - (n_a - v).e/c + |e x n_a|^2/(c (R + R_a - n_a.e))
// The bracket is precomputed per point in FP64 (dtau) and is small; the other
// terms are small because n_a ~ v for forward observers.
//
// Field (all FP32, per pixel and point), with W = beta_hat x N, c1 = 1 + beta_hat.N:
//    kappa = 1 - n.beta = eps + |beta| |W|^2 / c1,           eps = 1 - |beta|
//    N - beta = W x (N + beta_hat) / c1 + beta_hat * eps
//    E = (N-beta) scale/(gamma^2 R^2 kappa^3) + N x ((N-beta) x beta') scale/(c R kappa^3)
//    B c = N x E   (1/c applied in the FP64 reduction)
#include <cuda_runtime.h>

#include "lw_common.cuh"

namespace teufel {

// ---------------------------------------------------------------------------
// Per-point preparation (pixel independent), run once after upload
// ---------------------------------------------------------------------------
__global__ void prep_particles_kernel(DevTraj tr, double4_32a* vhat) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= tr.n_particles) return;
    int64_t o = tr.offsets[m], n = tr.offsets[m + 1] - o;
    double4_32a v = make_double4_32a(0.0, 0.0, 1.0, 0.0);
    if (n >= 2) {
        double4_32a a = tr.tx[o], b = tr.tx[o + n - 1];
        double dx = b.y - a.y, dy = b.z - a.z, dz = b.w - a.w;
        double L = sqrt(dx * dx + dy * dy + dz * dz);
        if (L > 0.0) v = make_double4_32a(dx / L, dy / L, dz / L, 0.0);
        // Arrival times increase along the trajectory for every observer when
        // time increases and every chord is slower than light (triangle
        // inequality); the range bisection relies on it.
        bool mono = true;
        for (int64_t i = o; i + 1 < o + n && mono; i++) {
            double4_32a p = tr.tx[i], q = tr.tx[i + 1];
            double ddt = q.x - p.x;
            double ex = q.y - p.y, ey = q.z - p.z, ez = q.w - p.w;
            double cd = kC * ddt;
            mono = (ddt > 0.0) && (ex * ex + ey * ey + ez * ez < 0.999999 * cd * cd);
        }
        v.w = mono ? 1.0 : 0.0;
    }
    vhat[m] = v;
}

__global__ void prep_points_kernel(DevTraj tr, float4* q0, float4* q1, float4* q2) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= tr.n_points) return;
    // particle of point i
    int lo = 0, hi = tr.n_particles - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (tr.offsets[mid] <= i) lo = mid; else hi = mid - 1;
    }
    int m = lo;
    int64_t o = tr.offsets[m];
    int64_t ia = o + ((i - o) & ~(int64_t)(kSegLen - 1));
    double4_32a p = tr.tx[i], a = tr.tx[ia];
    double4_32a v = tr.vhat[m];
    double ex = p.y - a.y, ey = p.z - a.z, ez = p.w - a.w;
    double ve = v.x * ex + v.y * ey + v.z * ez;
    double dtau = (p.x - a.x) - ve / kC;
    q0[i] = make_float4((float)ex, (float)ey, (float)ez, (float)dtau);
    double4_32a bg = tr.pp[i], ac = tr.aa[i];
    double P = sqrt(bg.x * bg.x + bg.y * bg.y + bg.z * bg.z);
    double gamma = sqrt(P * P + 1.0);
    double bx = v.x, by = v.y, bz = v.z, eps = 1.0;
    if (P > 0.0) {
        bx = bg.x / P;
        by = bg.y / P;
        bz = bg.z / P;
        eps = 1.0 / (gamma * (gamma + P));  // 1 - |beta| without cancellation
    }
    q1[i] = make_float4((float)bx, (float)by, (float)bz, (float)eps);
    double scale = field_scale(tr.charge[m]);
    double sa = scale / (gamma * kC);
    q2[i] = make_float4((float)(ac.x * sa), (float)(ac.y * sa), (float)(ac.z * sa),
                        (float)(scale / (gamma * gamma)));
}

// Error-bound data of each segment: max |dtau|, max |v.e|, max |e_perp|, max |e|.
__global__ void prep_segments_kernel(DevTraj tr, float4* segb) {
    int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= tr.n_segments) return;
    int m = particle_of_segment(tr.seg_offsets, tr.n_particles, g);
    int64_t o = tr.offsets[m], n = tr.offsets[m + 1] - o;
    int64_t first = o + (g - tr.seg_offsets[m]) * kSegLen;
    int64_t last = first + kSegLen;  // the next anchor closes the last step
    if (last > o + n - 1) last = o + n - 1;
    double4_32a a = tr.tx[first];
    double4_32a v = tr.vhat[m];
    double T = 0, Ez = 0, Ep = 0, Em = 0;
    for (int64_t i = first; i <= last; i++) {
        double4_32a p = tr.tx[i];
        double ex = p.y - a.y, ey = p.z - a.z, ez = p.w - a.w;
        double ve = v.x * ex + v.y * ey + v.z * ez;
        double dtau = (p.x - a.x) - ve / kC;
        double px = ex - ve * v.x, py = ey - ve * v.y, pz = ez - ve * v.z;
        T = fmax(T, fabs(dtau));
        Ez = fmax(Ez, fabs(ve));
        Ep = fmax(Ep, sqrt(px * px + py * py + pz * pz));
        Em = fmax(Em, sqrt(ex * ex + ey * ey + ez * ez));
    }
    segb[g] = make_float4((float)T * 1.0001f, (float)Ez * 1.0001f, (float)Ep * 1.0001f,
                          (float)Em * 1.0001f);
}

cudaError_t launch_prep_points(const DevTraj& tr, cudaStream_t s) {
    if (tr.n_particles > 0) {
        prep_particles_kernel<<<(tr.n_particles + 127) / 128, 128, 0, s>>>(
            tr, const_cast<double4_32a*>(tr.vhat));
    }
    if (tr.n_points > 0) {
        unsigned blocks = (unsigned)((tr.n_points + 255) / 256);
        prep_points_kernel<<<blocks, 256, 0, s>>>(tr, const_cast<float4*>(tr.q0),
                                                  const_cast<float4*>(tr.q1),
                                                  const_cast<float4*>(tr.q2));
    }
    if (tr.n_segments > 0) {
        unsigned blocks = (unsigned)((tr.n_segments + 127) / 128);
        prep_segments_kernel<<<blocks, 128, 0, s>>>(tr, const_cast<float4*>(tr.segb));
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Anchor and point evaluation (shared by the main kernel and the decision
// record used by the bin-index parity tests)
// ---------------------------------------------------------------------------
struct PixelCtx {
    double3 P;
    Window w;
    double inv_dt, inv_cdt;
    float kdt, kcd;
};

__device__ __forceinline__ PixelCtx make_pixel(double3 P, double t0, double dt, int nt) {
    PixelCtx c;
    c.P = P;
    c.w = make_window(t0, dt, nt);
    c.inv_dt = 1.0 / dt;
    c.inv_cdt = 1.0 / (kC * dt);
    c.kdt = (float)c.inv_dt;
    c.kcd = (float)c.inv_cdt;
    return c;
}

struct Anchor {
    long long B;     // floor of the anchor's (ts - t0)/dt
    float frac;      // the rest, in [0, 1)
    float Dx, Dy, Dz;
    float nx, ny, nz;
    float mx, my, mz;  // n_a - v
    float R;
    float band;      // half-width of the ambiguity band around half-integers [bins]
    bool exact;      // segment too coarse for the FP32 estimate
};

__device__ __forceinline__ void make_anchor(Anchor& A, const DevTraj& tr, int64_t ia, int64_t seg,
                                            const PixelCtx& px, double4_32a v) {
    double4_32a a = tr.tx[ia];
    double Dx = px.P.x - a.y, Dy = px.P.y - a.z, Dz = px.P.z - a.w;
    double R2 = fma(Dx, Dx, fma(Dy, Dy, Dz * Dz));
    double R = sqrt(R2);
    double iR = 1.0 / R;
    double nx = Dx * iR, ny = Dy * iR, nz = Dz * iR;
    double u = fma(a.x - px.w.t0, px.inv_dt, R * px.inv_cdt);
    u = fmax(-1.0e15, fmin(u, 1.0e15));
    double fl = floor(u);
    A.B = (long long)fl;
    A.frac = (float)(u - fl);
    A.Dx = (float)Dx;
    A.Dy = (float)Dy;
    A.Dz = (float)Dz;
    A.nx = (float)nx;
    A.ny = (float)ny;
    A.nz = (float)nz;
    A.mx = (float)(nx - v.x);
    A.my = (float)(ny - v.y);
    A.mz = (float)(nz - v.z);
    A.R = (float)R;
    // error bound of the FP32 estimate (16 x 2^-24 x the magnitudes entering it)
    double cm1 = fma(nx, v.x, fma(ny, v.y, nz * v.z)) - 1.0;  // cos(theta) - 1
    float c1 = (float)(-cm1);
    float st = sqrtf(fmaxf(0.0f, c1 * (2.0f - c1)));
    float4 sb = tr.segb[seg];
    float ep = sb.z + st * sb.y;
    float span = sb.x * px.kdt + (c1 * sb.y + st * sb.z + __fdividef(ep * ep, A.R)) * px.kcd +
                 2.0f;
    // the reference's own rounding of ts and of tmin/tmax, in bins
    float refb = (float)((fabs(a.x) + R / kC + fabs(px.w.t0)) * px.inv_dt * 1.0e-15);
    A.band = 16.0f * 5.9604645e-8f * span + refb;
    A.exact = !(A.band < 0.0625f);
}

struct PointState {
    float off;   // (ts - t0)/dt - B
    int idx;     // bin index (clamped to [-2, nt+1])
    int flags;   // kLeTmin | kLtTmax | kExact
    float f[6];  // Ex, Ey, Ez, c*Bx, c*By, c*Bz
};

__device__ __forceinline__ void eval_time(PointState& S, const DevTraj& tr, int64_t i,
                                          const Anchor& A, float4 q0, float3 v,
                                          const PixelCtx& px, float R) {
    float ex = q0.x, ey = q0.y, ez = q0.z;
    float nme = A.mx * ex + A.my * ey + A.mz * ez;
    float ve = v.x * ex + v.y * ey + v.z * ez;
    float L = A.R - ve - nme;
    float cx = ey * A.nz - ez * A.ny, cy = ez * A.nx - ex * A.nz, cz = ex * A.ny - ey * A.nx;
    float G = __fdividef(cx * cx + cy * cy + cz * cz, R + L);
    float du = q0.w * px.kdt - (nme - G) * px.kcd;
    float off = A.frac + du;
    float vv = off + 0.5f;
    float fk = floorf(vv);
    float fr = vv - fk;
    if (A.exact || fr < A.band || fr > 1.0f - A.band) {
        double ts = exact_retarded_time(tr.tx[i], px.P);
        S.idx = exact_bin(ts, px.w);
        S.flags = exact_flags(ts, px.w);
        S.off = (float)((ts - px.w.t0) * px.inv_dt - (double)A.B);
    } else {
        long long k = A.B + (long long)fk;
        k = k < -2 ? -2 : (k > px.w.nt + 1 ? px.w.nt + 1 : k);
        S.idx = (int)k;
        S.flags = (k < 0 ? kLeTmin : 0) | (k < px.w.nt ? kLtTmax : 0);
        S.off = off;
    }
}

__device__ __forceinline__ void eval_point(PointState& S, const DevTraj& tr, int64_t i,
                                           const Anchor& A, float3 v, const PixelCtx& px) {
    float4 a = __ldg(tr.q0 + i);
    float4 b = __ldg(tr.q1 + i);
    float4 c = __ldg(tr.q2 + i);
    float Dx = A.Dx - a.x, Dy = A.Dy - a.y, Dz = A.Dz - a.z;
    float R2 = Dx * Dx + Dy * Dy + Dz * Dz;
    float iR = rsqrtf(R2);
    float R = R2 * iR;
    float Nx = Dx * iR, Ny = Dy * iR, Nz = Dz * iR;
    eval_time(S, tr, i, A, a, v, px, R);
    // kappa = 1 - n.beta in split form
    float Wx = b.y * Nz - b.z * Ny, Wy = b.z * Nx - b.x * Nz, Wz = b.x * Ny - b.y * Nx;
    float s2 = Wx * Wx + Wy * Wy + Wz * Wz;
    float rc1 = __fdividef(1.0f, 1.0f + (b.x * Nx + b.y * Ny + b.z * Nz));
    float kappa = b.w + (1.0f - b.w) * s2 * rc1;
    // N - beta = W x (N + beta_hat) / c1 + beta_hat * eps
    float Sx = Nx + b.x, Sy = Ny + b.y, Sz = Nz + b.z;
    float mbx = (Wy * Sz - Wz * Sy) * rc1 + b.x * b.w;
    float mby = (Wz * Sx - Wx * Sz) * rc1 + b.y * b.w;
    float mbz = (Wx * Sy - Wy * Sx) * rc1 + b.z * b.w;
    float rk = __fdividef(1.0f, kappa);
    float rk3 = rk * rk * rk;
    float cvel = c.w * iR * iR * rk3;
    float cacc = iR * rk3;
    // (N - beta) x beta'
    float px_ = mby * c.z - mbz * c.y, py_ = mbz * c.x - mbx * c.z, pz_ = mbx * c.y - mby * c.x;
    // N x that
    float ax = Ny * pz_ - Nz * py_, ay = Nz * px_ - Nx * pz_, az = Nx * py_ - Ny * px_;
    float Ex = mbx * cvel + ax * cacc;
    float Ey = mby * cvel + ay * cacc;
    float Ez = mbz * cvel + az * cacc;
    S.f[0] = Ex;
    S.f[1] = Ey;
    S.f[2] = Ez;
    S.f[3] = Ny * Ez - Nz * Ey;
    S.f[4] = Nz * Ex - Nx * Ez;
    S.f[5] = Nx * Ey - Ny * Ex;
}

// ---------------------------------------------------------------------------
// Main kernel
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128, 4)
    lw_fp32_kernel(DevTraj tr, DevScreen sc, DevWork wk) {
    const int slot = blockIdx.y;
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = pix < sc.np;
    const int pc = active ? pix : sc.np - 1;
    const double3 P = make_double3(sc.pix_pos[3 * pc], sc.pix_pos[3 * pc + 1],
                                   sc.pix_pos[3 * pc + 2]);
    const PixelCtx px = make_pixel(P, sc.pix_t0[pc], sc.dt, sc.nt);
    BinSink<float, 6> sink;
    sink.init(static_cast<float*>(wk.scratch) + (int64_t)slot * wk.slot_stride +
                  (int64_t)pc * sc.nt * 6,
              sc.nt);
    const int64_t g0 = wk.slot_seg[slot], g1 = wk.slot_seg[slot + 1];
    int m = g0 < g1 ? particle_of_segment(tr.seg_offsets, tr.n_particles, g0) : tr.n_particles;
    unsigned long long inwin = 0, nfb = 0;
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
        const double4_32a vd = tr.vhat[m];
        int first = st_lo, last = st_hi - 1;
        if (vd.w != 0.0) inwindow_steps(tr.tx + po, st_lo, st_hi, P, px.w, &first, &last);
        if (!active) last = first - 1;
        // align every lane's start to a segment boundary so that all lanes
        // change anchors on the same iteration
        int start = first & ~(kSegLen - 1);
        if (start < st_lo) start = st_lo;
        const int trips = last >= first ? last - start + 1 : 0;
        const int max_trips = warp_max(trips);
        if (max_trips == 0) continue;
        if (trips == 0) start = st_lo;
        const float3 v = make_float3((float)vd.x, (float)vd.y, (float)vd.z);
        Anchor A;
        make_anchor(A, tr, po + start, sb + (start >> kSegShift), px, vd);
        PointState p1, p2;
        eval_point(p1, tr, po + start, A, v, px);
        nfb += (p1.flags & kExact) ? 1 : 0;
        for (int j = 0; j < max_trips; ++j) {
            const int i2 = start + j + 1;
            const bool live = j < trips;
            if ((i2 & (kSegLen - 1)) == 0) {
                const int i2c = i2 < npm ? i2 : ((npm - 1) & ~(kSegLen - 1));
                Anchor An;
                make_anchor(An, tr, po + i2c, sb + (i2c >> kSegShift), px, vd);
                p1.off -= (float)(An.B - A.B);
                A = An;
            }
            if (live) {
                eval_point(p2, tr, po + i2, A, v, px);
                nfb += (p2.flags & kExact) ? 1 : 0;
                Geo32 geo{A.B};
                if (deposit_step<Ops32>(p1.off, p2.off, p1.idx, p1.flags, p2.idx, p2.flags, p1.f,
                                        p2.f, geo, sc.nt, sink))
                    inwin++;
                p1 = p2;
            }
        }
    }
    sink.flush();
    if (sink.err) atomicOr(wk.status, sink.err);
    // statistics: one atomic per warp
    inwin = warp_sum_u64(inwin);
    nfb = warp_sum_u64(nfb);
    if ((threadIdx.x & 31) == 0 && wk.counters) {
        if (inwin) atomicAdd(wk.counters, inwin);
        if (nfb) atomicAdd(wk.counters + 1, nfb);
    }
}

cudaError_t launch_fp32(const DevTraj& tr, const DevScreen& sc, const DevWork& w, int threads,
                        cudaStream_t s) {
    if (threads != 128) threads = 128;
    dim3 grid((sc.np + threads - 1) / threads, w.n_slots);
    lw_fp32_kernel<<<grid, threads, 0, s>>>(tr, sc, w);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Decision record for the parity tests: one thread per point of particle m
// ---------------------------------------------------------------------------
__global__ void point_decisions_kernel(DevTraj tr, int m, double3 P, double t0, double dt,
                                       int nt, int64_t* idx, int* flags, double* u_est) {
    int64_t o = tr.offsets[m];
    int n = (int)(tr.offsets[m + 1] - o);
    int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n) return;
    PixelCtx px = make_pixel(P, t0, dt, nt);
    double4_32a vd = tr.vhat[m];
    float3 v = make_float3((float)vd.x, (float)vd.y, (float)vd.z);
    int a = l & ~(kSegLen - 1);
    Anchor A;
    make_anchor(A, tr, o + a, tr.seg_offsets[m] + (a >> kSegShift), px, vd);
    PointState S;
    eval_point(S, tr, o + l, A, v, px);
    idx[l] = S.idx;
    flags[l] = S.flags;
    // the FP32 estimate itself, for error-bound checks
    float4 q = tr.q0[o + l];
    float Dx = A.Dx - q.x, Dy = A.Dy - q.y, Dz = A.Dz - q.z;
    float R2 = Dx * Dx + Dy * Dy + Dz * Dz;
    float R = R2 * rsqrtf(R2);
    Anchor Ae = A;
    Ae.exact = false;
    Ae.band = -1.0f;
    PointState T;
    eval_time(T, tr, o + l, Ae, q, v, px, R);
    u_est[l] = (double)A.B + (double)T.off;
}

cudaError_t launch_point_decisions(const DevTraj& tr, int m, double3 pos, double t0, double dt,
                                   int nt, int64_t* idx, int* flags, double* u_est,
                                   unsigned int* status, cudaStream_t s) {
    (void)status;
    int64_t n = 0;
    cudaMemcpyAsync(&n, tr.offsets + m + 1, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    int64_t o = 0;
    cudaMemcpyAsync(&o, tr.offsets + m, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    n -= o;
    if (n <= 0) return cudaGetLastError();
    point_decisions_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(tr, m, pos, t0, dt, nt,
                                                                       idx, flags, u_est);
    return cudaGetLastError();
}

}  // namespace teufel
