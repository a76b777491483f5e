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
    q0[i] = make_float4((float)(p.y - a.y), (float)(p.z - a.z), (float)(p.w - a.w), (float)ddt);
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
    q1[i] = make_float4((float)bx, (float)by, (float)bz, (float)eps);
    double scale = field_scale(tr.charge[m]);
    double sa = scale / (gamma * kC);
    q2[i] = make_float4((float)(ac.x * sa), (float)(ac.y * sa), (float)(ac.z * sa),
                        (float)(scale / (gamma * gamma)));
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
                                                  const_cast<float4*>(tr.q2),
                                                  const_cast<float4*>(tr.q3));
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Double-float helpers (error-free transformations)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
    s = a + b;
    double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void two_prod(double a, double b, double& p, double& e) {
    p = a * b;
    e = fma(a, b, -p);
}

// ---------------------------------------------------------------------------
// Pixel, anchor and point evaluation (shared by the main kernel and the
// decision record used by the bin-index parity tests)
// ---------------------------------------------------------------------------
struct PixelCtx {
    double3 P;
    double3 Ph;   // P / |P|
    double Pn;    // |P|
    double Tp;    // |P|/c - t0, formed in double-float
    Window w;
    double inv_dt;
    float kdt;    // 1/dt
    float refb0;  // the reference's rounding of t0 and of the flight time [bins]
};

__device__ __forceinline__ PixelCtx make_pixel(double3 P, double t0, double dt, int nt) {
    PixelCtx c;
    c.P = P;
    c.w = make_window(t0, dt, nt);
    c.inv_dt = 1.0 / dt;
    c.kdt = (float)c.inv_dt;
    // |P|^2 and |P| in double-float
    double s, e, p, q, e2;
    two_prod(P.x, P.x, s, e);
    two_prod(P.y, P.y, p, q);
    two_sum(s, p, s, e2);
    e += q + e2;
    two_prod(P.z, P.z, p, q);
    two_sum(s, p, s, e2);
    e += q + e2;
    double n_hi = sqrt(s);
    double n_lo = n_hi > 0.0 ? (fma(-n_hi, n_hi, s) + e) / (2.0 * n_hi) : 0.0;
    c.Pn = n_hi;
    double r = n_hi > 0.0 ? 1.0 / n_hi : 0.0;
    c.Ph = make_double3(P.x * r, P.y * r, P.z * r);
    // |P|/c - t0 with 1/c as a double-float
    const double ic_hi = 1.0 / kC;
    const double ic_lo = fma(-ic_hi, kC, 1.0) / kC;
    double qh, ql;
    two_prod(n_hi, ic_hi, qh, ql);
    ql += n_hi * ic_lo + n_lo * ic_hi;
    double d, de;
    two_sum(qh, -t0, d, de);
    c.Tp = d + (de + ql);
    // the reference rounds |P - x|/c (~ |P|/c) and t + R/c; t0 and tmin/tmax
    c.refb0 = (float)((n_hi / kC * 4.5e-16 + fabs(t0) * 2.3e-16) * c.inv_dt);
    return c;
}

struct Anchor {
    long long B;   // floor of the anchor's (ts - t0)/dt
    float frac;    // the rest, in [0, 1)
    float Dx, Dy, Dz;
    float err;     // bound on the anchor's error plus the reference's rounding [bins]
};

__device__ __forceinline__ void make_anchor(Anchor& A, const DevTraj& tr, int64_t ia,
                                            const PixelCtx& px) {
    const double4_32a a = tr.tx[ia];
    const double Dx = px.P.x - a.y, Dy = px.P.y - a.z, Dz = px.P.z - a.w;
    const double pa = fma(px.Ph.x, a.y, fma(px.Ph.y, a.z, px.Ph.z * a.w));  // P^.x
    const double L = px.Pn - pa;
    const double cx = a.z * px.Ph.z - a.w * px.Ph.y;
    const double cy = a.w * px.Ph.x - a.y * px.Ph.z;
    const double cz = a.y * px.Ph.y - a.z * px.Ph.x;
    const double g2 = fma(cx, cx, fma(cy, cy, cz * cz));  // |x x P^|^2
    double G;
    if (L > 0.0 && g2 < 1.0e-4 * L * L) {
        // G = g2 / (L + sqrt(L^2 + g2)) as a series in q = g2/L^2
        double rL = (double)__frcp_rn((float)L);
        rL = rL * fma(-L, rL, 2.0);
        rL = rL * fma(-L, rL, 2.0);
        const double q = g2 * rL * rL;
        G = g2 * rL * fma(q, fma(q, 0.0625, -0.125), 0.5);
    } else {
        G = g2 / (L + sqrt(fma(L, L, g2)));
    }
    const double ic = 1.0 / kC;
    const double tau = fma(-pa, ic, a.x);  // t - P^.x / c
    double u = (px.Tp + tau + G * ic) * px.inv_dt;
    u = fmax(-1.0e15, fmin(u, 1.0e15));
    const double fl = floor(u);
    A.B = (long long)fl;
    A.frac = (float)(u - fl);
    A.Dx = (float)Dx;
    A.Dy = (float)Dy;
    A.Dz = (float)Dz;
    // our rounding: t, P^.x/c and their sum, G/c, the sum with Tp, the scaling
    const float own = (float)((fabs(a.x) + fabs(pa) * ic + fabs(px.Tp) + G * ic) * px.inv_dt *
                              4.5e-16) +
                      (float)(fabs(u) * 4.5e-16) + 1.0e-7f;
    A.err = own + px.refb0 + (float)(fabs(a.x) * px.inv_dt * 4.5e-16);
}

struct PointState {
    long long ui;  // nearest integer to (ts - t0)/dt (unclamped)
    float r;       // (ts - t0)/dt - ui
    int idx;       // bin index round((ts-t0)/dt), clamped to [-2, nt+1]
    int flags;     // kLeTmin | kLtTmax | kExact
    float Nx, Ny, Nz;
    float f[6];    // Ex, Ey, Ez, c*Bx, c*By, c*Bz
};

// Field of one point from its anchor-relative position.
__device__ __forceinline__ void point_field(PointState& S, float4 a, float4 b, float4 c,
                                            const Anchor& A) {
    const float Dx = A.Dx - a.x, Dy = A.Dy - a.y, Dz = A.Dz - a.z;
    const float R2 = Dx * Dx + Dy * Dy + Dz * Dz;
    const float iR = rsqrtf(R2);
    const float Nx = Dx * iR, Ny = Dy * iR, Nz = Dz * iR;
    S.Nx = Nx;
    S.Ny = Ny;
    S.Nz = Nz;
    // kappa = 1 - n.beta in split form
    const float Wx = b.y * Nz - b.z * Ny, Wy = b.z * Nx - b.x * Nz, Wz = b.x * Ny - b.y * Nx;
    const float s2 = Wx * Wx + Wy * Wy + Wz * Wz;
    const float rc1 = __fdividef(1.0f, 1.0f + (b.x * Nx + b.y * Ny + b.z * Nz));
    const float kappa = b.w + (1.0f - b.w) * s2 * rc1;
    // N - beta = W x (N + beta_hat) / c1 + beta_hat * eps
    const float Sx = Nx + b.x, Sy = Ny + b.y, Sz = Nz + b.z;
    const float mbx = (Wy * Sz - Wz * Sy) * rc1 + b.x * b.w;
    const float mby = (Wz * Sx - Wx * Sz) * rc1 + b.y * b.w;
    const float mbz = (Wx * Sy - Wy * Sx) * rc1 + b.z * b.w;
    const float rk = __fdividef(1.0f, kappa);
    const float rk3 = rk * rk * rk;
    const float cvel = c.w * iR * iR * rk3;
    const float cacc = iR * rk3;
    // N x ((N - beta) x beta')
    const float px_ = mby * c.z - mbz * c.y, py_ = mbz * c.x - mbx * c.z, pz_ = mbx * c.y - mby * c.x;
    const float ax = Ny * pz_ - Nz * py_, ay = Nz * px_ - Nx * pz_, az = Nx * py_ - Ny * px_;
    const float Ex = mbx * cvel + ax * cacc;
    const float Ey = mby * cvel + ay * cacc;
    const float Ez = mbz * cvel + az * cacc;
    S.f[0] = Ex;
    S.f[1] = Ey;
    S.f[2] = Ez;
    S.f[3] = Ny * Ez - Nz * Ey;
    S.f[4] = Nz * Ex - Nx * Ez;
    S.f[5] = Nx * Ey - Ny * Ex;
}

// Arrival increment of the step from point 1 to point 2 [bins]:
//   dt (1 - |beta_c| + |beta_c| (1 - |n_m|) + |beta_c| |n_m| (1 - cos theta))
// with n_m along N1 + N2, 1 - |n_m| = |N1 - N2|^2 / 8 to leading order, and
// 1 - cos theta = |beta_c x s|^2 / (|s| (|s| + beta_c.s)), s = N1 + N2.
__device__ __forceinline__ float step_increment(const PointState& p1, const PointState& p2,
                                                float4 chord, float dtstep, float kdt) {
    const float sx = p1.Nx + p2.Nx, sy = p1.Ny + p2.Ny, sz = p1.Nz + p2.Nz;
    const float dx = p1.Nx - p2.Nx, dy = p1.Ny - p2.Ny, dz = p1.Nz - p2.Nz;
    const float wx = chord.y * sz - chord.z * sy;
    const float wy = chord.z * sx - chord.x * sz;
    const float wz = chord.x * sy - chord.y * sx;
    const float w2 = wx * wx + wy * wy + wz * wz;
    const float ss = sx * sx + sy * sy + sz * sz;
    const float rs = rsqrtf(ss);
    const float sn = ss * rs;  // |s|
    const float bs = chord.x * sx + chord.y * sy + chord.z * sz;
    const float one_m_cos = __fdividef(w2, sn * (sn + bs));
    const float one_m_n = 0.125f * (dx * dx + dy * dy + dz * dz);
    const float beta = 1.0f - chord.w;
    const float kap = chord.w + beta * (one_m_n + one_m_cos);
    return dtstep * kdt * kap;
}

// Bin decision from (ui, r); falls back to the reference's exact FP64
// evaluation when r is within `band` of +-1/2.
__device__ __forceinline__ void decide(PointState& S, float band, const DevTraj& tr, int64_t i,
                                       const PixelCtx& px) {
    const float d = 0.5f - fabsf(S.r);  // distance to the nearest half-integer
    if (d <= band) {
        const double ts = exact_retarded_time(tr.tx[i], px.P);
        S.idx = exact_bin(ts, px.w);
        S.flags = exact_flags(ts, px.w);
        // continue from the exact value
        const double u = (ts - px.w.t0) * px.inv_dt;
        const double k = floor(u + 0.5);
        S.ui = (long long)fmax(-1.0e15, fmin(k, 1.0e15));
        S.r = (float)(u - (double)S.ui);
    } else {
        long long k = S.ui;
        const int nt = px.w.nt;
        k = k < -2 ? -2 : (k > nt + 1 ? nt + 1 : k);
        S.idx = (int)k;
        S.flags = (k < 0 ? kLeTmin : 0) | (k < nt ? kLtTmax : 0);
    }
}

// Start a compensated arrival chain at an anchor point.
__device__ __forceinline__ void start_chain(PointState& S, const Anchor& A) {
    const float k = rintf(A.frac);  // 0 or 1
    S.ui = A.B + (long long)k;
    S.r = A.frac - k;
}

// ---------------------------------------------------------------------------
// The deposit of one step in bin units, from (ui, r) arrival coordinates;
// the same branch structure and weights as deposit_step (lw_common.cuh),
// src/particle.cpp:786-865.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float dist(long long a, long long b) { return (float)(a - b); }

template <class Sink>
__device__ __forceinline__ bool deposit_step32(const PointState& p1, const PointState& p2, int nt,
                                               Sink& sink) {
    if ((p2.flags & kLeTmin) || !(p1.flags & kLtTmax)) return false;
    const float dts = dist(p2.ui, p1.ui) + (p2.r - p1.r);
    const float rd = __fdividef(1.0f, dts);
    float field[6];
    int idx2 = p2.idx > nt ? nt : p2.idx;
    if (p1.flags & kLeTmin) {
        for (int k = 0; k < idx2; k++) {
            const float w1 = (dist(p2.ui, k) + p2.r) * rd;
            const float w2 = (dist(k, p1.ui) - p1.r) * rd;
#pragma unroll
            for (int c = 0; c < 6; c++) field[c] = p1.f[c] * w1 + p2.f[c] * w2;
            sink.add(k, field);
        }
        if (idx2 < nt) {
            const float a2 = dist(p2.ui, idx2) + p2.r + 0.5f;  // ts2 - t_start
            const float a1 = dist(idx2, p1.ui) - 0.5f - p1.r;  // t_start - ts1
            const float w1 = a2 * rd, w2 = a1 * rd, wb = 0.5f * a2;
#pragma unroll
            for (int c = 0; c < 6; c++) field[c] = (p1.f[c] * w1 + p2.f[c] * (w2 + 1.0f)) * wb;
            sink.add(idx2, field);
        }
    } else {
        const int idx1 = p1.idx;
        if (idx1 == idx2) {
            const float wb = 0.5f * dts;
#pragma unroll
            for (int c = 0; c < 6; c++) field[c] = (p1.f[c] + p2.f[c]) * wb;
            sink.add(idx1, field);
        } else {
            {
                const float b2 = dist(p2.ui, idx1) - 0.5f + p2.r;  // ts2 - t_end
                const float b1 = dist(idx1, p1.ui) + 0.5f - p1.r;  // t_end - ts1
                const float w1 = b2 * rd, w2 = b1 * rd, wb = 0.5f * b1;
#pragma unroll
                for (int c = 0; c < 6; c++) field[c] = (p1.f[c] * (1.0f + w1) + p2.f[c] * w2) * wb;
                sink.add(idx1, field);
            }
            for (int k = idx1 + 1; k < idx2; k++) {
                const float w1 = (dist(p2.ui, k) + p2.r) * rd;
                const float w2 = (dist(k, p1.ui) - p1.r) * rd;
#pragma unroll
                for (int c = 0; c < 6; c++) field[c] = p1.f[c] * w1 + p2.f[c] * w2;
                sink.add(k, field);
            }
            if (idx2 < nt) {
                const float a2 = dist(p2.ui, idx2) + p2.r + 0.5f;
                const float a1 = dist(idx2, p1.ui) - 0.5f - p1.r;
                const float w1 = a2 * rd, w2 = a1 * rd, wb = 0.5f * a2;
#pragma unroll
                for (int c = 0; c < 6; c++) field[c] = (p1.f[c] * w1 + p2.f[c] * (w2 + 1.0f)) * wb;
                sink.add(idx2, field);
            }
        }
    }
    return true;
}

// ---------------------------------------------------------------------------
// Main kernel
// ---------------------------------------------------------------------------
constexpr float kChainRel = 1.0e-6f;  // bound on the relative error of one FP32 increment

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
        int first = st_lo, last = st_hi - 1;
        if (tr.vhat[m].w != 0.0) inwindow_steps(tr.tx + po, st_lo, st_hi, P, px.w, &first, &last);
        if (!active) last = first - 1;
        // align every lane's start to a segment boundary so that all lanes
        // change anchors on the same iteration
        int start = first & ~(kSegLen - 1);
        if (start < st_lo) start = st_lo;
        const int trips = last >= first ? last - start + 1 : 0;
        const int max_trips = warp_max(trips);
        if (max_trips == 0) continue;
        if (trips == 0) start = st_lo;
        Anchor A;
        make_anchor(A, tr, po + start, px);
        PointState p1, p2;
        point_field(p1, __ldg(tr.q0 + po + start), __ldg(tr.q1 + po + start),
                    __ldg(tr.q2 + po + start), A);
        start_chain(p1, A);
        decide(p1, A.err, tr, po + start, px);
        nfb += (p1.flags & kExact) ? 1 : 0;
        float comp = 0.0f, chain_err = 0.0f;
        for (int j = 0; j < max_trips; ++j) {
            const int i2 = start + j + 1;
            const bool live = j < trips;
            if ((i2 & (kSegLen - 1)) == 0) {
                const int i2c = i2 < npm ? i2 : ((npm - 1) & ~(kSegLen - 1));
                make_anchor(A, tr, po + i2c, px);
            }
            if (live) {
                const int64_t g1i = po + i2 - 1, g2i = po + i2;
                const float4 q0a = __ldg(tr.q0 + g1i);
                point_field(p2, __ldg(tr.q0 + g2i), __ldg(tr.q1 + g2i), __ldg(tr.q2 + g2i), A);
                if ((i2 & (kSegLen - 1)) == 0) {
                    start_chain(p2, A);
                    comp = 0.0f;
                    chain_err = 0.0f;
                } else {
                    const float du = step_increment(p1, p2, __ldg(tr.q3 + g1i), q0a.w, px.kdt);
                    // compensated sum r2 = r1 + du, then renormalize
                    const float y = du - comp;
                    const float t = p1.r + y;
                    comp = (t - p1.r) - y;
                    const float k = rintf(t);
                    p2.r = t - k;
                    p2.ui = p1.ui + (long long)k;
                    chain_err += fabsf(du) * kChainRel + 1.0e-7f;
                }
                decide(p2, A.err + chain_err, tr, g2i, px);
                nfb += (p2.flags & kExact) ? 1 : 0;
                if (deposit_step32(p1, p2, sc.nt, sink)) inwin++;
                p1 = p2;
            }
        }
    }
    sink.flush();
    if (sink.err) atomicOr(wk.status, sink.err);
    // statistics: one atomic per warp
    inwin = warp_sum_u64(inwin);
    nfb = warp_sum_u64(nfb);
    unsigned long long nadd = warp_sum_u64(sink.n_add);
    if ((threadIdx.x & 31) == 0 && wk.counters) {
        if (inwin) atomicAdd(wk.counters, inwin);
        if (nfb) atomicAdd(wk.counters + 1, nfb);
        if (nadd) atomicAdd(wk.counters + 2, nadd);
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
    BinSink<float, 6> sink;
    sink.init(trace32, nt);
    for (int m = 0; m < n_part; m++) {
        const int64_t o = offs[m], n = offs[m + 1] - o;
        PointState p1, p2;
        for (int64_t s = 0; s < n; s++) {
            const double t = ts[o + s];
            const double u = (t - t0) / dt;
            const double k = floor(u + 0.5);
            p2.ui = (long long)fmax(-1.0e15, fmin(k, 1.0e15));
            p2.r = (float)(u - (double)p2.ui);
            p2.idx = exact_bin(t, w);
            p2.flags = exact_flags(t, w);
            for (int c = 0; c < 6; c++) p2.f[c] = (float)f[6 * (o + s) + c];
            if (s > 0) deposit_step32(p1, p2, nt, sink);
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
// m walks its points exactly as the main kernel does.
// ---------------------------------------------------------------------------
__global__ void point_decisions_kernel(DevTraj tr, int m, double3 P, double t0, double dt,
                                       int nt, int64_t* idx, int* flags, double* u_est) {
    const int64_t o = tr.offsets[m];
    const int n = (int)(tr.offsets[m + 1] - o);
    const int seg = blockIdx.x * blockDim.x + threadIdx.x;
    const int start = seg << kSegShift;
    if (start >= n) return;
    const PixelCtx px = make_pixel(P, t0, dt, nt);
    Anchor A;
    make_anchor(A, tr, o + start, px);
    PointState p1, p2;
    point_field(p1, tr.q0[o + start], tr.q1[o + start], tr.q2[o + start], A);
    start_chain(p1, A);
    u_est[start] = (double)p1.ui + (double)p1.r;
    decide(p1, A.err, tr, o + start, px);
    idx[start] = p1.idx;
    flags[start] = p1.flags;
    float comp = 0.0f, chain_err = 0.0f;
    const int end = min(start + kSegLen, n - 1);  // the next anchor belongs to the next thread
    for (int i2 = start + 1; i2 < n && i2 < start + kSegLen; i2++) {
        point_field(p2, tr.q0[o + i2], tr.q1[o + i2], tr.q2[o + i2], A);
        const float du = step_increment(p1, p2, tr.q3[o + i2 - 1], tr.q0[o + i2 - 1].w, px.kdt);
        const float y = du - comp;
        const float t = p1.r + y;
        comp = (t - p1.r) - y;
        const float k = rintf(t);
        p2.r = t - k;
        p2.ui = p1.ui + (long long)k;
        chain_err += fabsf(du) * kChainRel + 1.0e-7f;
        u_est[i2] = (double)p2.ui + (double)p2.r;
        decide(p2, A.err + chain_err, tr, o + i2, px);
        idx[i2] = p2.idx;
        flags[i2] = p2.flags;
        p1 = p2;
    }
    (void)end;
}

cudaError_t launch_point_decisions(const DevTraj& tr, int m, double3 pos, double t0, double dt,
                                   int nt, int64_t n_points, int64_t* idx, int* flags,
                                   double* u_est, cudaStream_t s) {
    if (n_points <= 0) return cudaSuccess;
    const int64_t nseg = (n_points + kSegLen - 1) / kSegLen;
    point_decisions_kernel<<<(unsigned)((nseg + 127) / 128), 128, 0, s>>>(tr, m, pos, t0, dt, nt,
                                                                         idx, flags, u_est);
    return cudaGetLastError();
}

}  // namespace teufel
