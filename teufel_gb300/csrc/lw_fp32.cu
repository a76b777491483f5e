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

// Arrival coordinates are held relative to the current anchor's integer bin
// B as (ki, r): (ts - t0)/dt = B + ki + r, |r| <= 1/2 normally.  B is kept
// within +-2^29 so that B + ki never overflows 32 bits; anchors farther out
// than that send every point of their segment through the exact path.
constexpr double kBinLimit = 536870912.0;  // 2^29

struct Anchor {
    long long B;   // floor of the anchor's (ts - t0)/dt, clamped to +-2^29
    int Bi;        // the same, as int
    float frac;    // the rest, in [0, 1)
    float Dx, Dy, Dz;
    float err;     // bound on the anchor's error plus the reference's rounding [bins]
};

__device__ __forceinline__ void make_anchor(Anchor& A, const double4_32a a, const PixelCtx& px) {
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
    const double u0 = (px.Tp + tau + G * ic) * px.inv_dt;
    const double u = fmax(-kBinLimit, fmin(u0, kBinLimit));
    const double fl = floor(u);
    A.B = (long long)fl;
    A.Bi = (int)fl;
    A.frac = (float)(u - fl);
    A.Dx = (float)Dx;
    A.Dy = (float)Dy;
    A.Dz = (float)Dz;
    // our rounding: t, P^.x/c and their sum, G/c, the sum with Tp, the scaling
    const float own = (float)((fabs(a.x) + fabs(pa) * ic + fabs(px.Tp) + G * ic) * px.inv_dt *
                              4.5e-16) +
                      (float)(fabs(u) * 4.5e-16) + 1.0e-7f;
    A.err = own + px.refb0 + (float)(fabs(a.x) * px.inv_dt * 4.5e-16);
    if (u != u0) A.err = 1.0f;  // clamped: resolve the segment exactly
}

struct PointState {
    int ki;        // integer part of (ts - t0)/dt - B
    float r;       // the rest
    int idx;       // bin index round((ts-t0)/dt), clamped to [-2, nt+1]
    int flags;     // kLeTmin | kLtTmax | kExact
    float dt;      // duration of the trajectory step that starts at this point
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
    S.dt = a.w;
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
    const float cacc = iR * rk3;
    const float cvel = c.w * iR * cacc;
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
// 1 - cos theta = |beta_c x s|^2 / (|s| (|s| + beta_c.s)), s = N1 + N2, |s| ~ 2
// (|s| = 2 - |N1 - N2|^2/4, and the FP32 normalisation of N is good to 1e-7).
__device__ __forceinline__ float step_increment(const PointState& p1, const PointState& p2,
                                                float4 chord, float kdt) {
    const float sx = p1.Nx + p2.Nx, sy = p1.Ny + p2.Ny, sz = p1.Nz + p2.Nz;
    const float dx = p1.Nx - p2.Nx, dy = p1.Ny - p2.Ny, dz = p1.Nz - p2.Nz;
    const float wx = chord.y * sz - chord.z * sy;
    const float wy = chord.z * sx - chord.x * sz;
    const float wz = chord.x * sy - chord.y * sx;
    const float w2 = wx * wx + wy * wy + wz * wz;
    const float bs = chord.x * sx + chord.y * sy + chord.z * sz;
    const float one_m_cos = __fdividef(w2, 4.0f + 2.0f * bs);
    const float one_m_n = 0.125f * (dx * dx + dy * dy + dz * dz);
    const float kap = chord.w + (1.0f - chord.w) * (one_m_n + one_m_cos);
    return p1.dt * kdt * kap;
}

// Advance the compensated arrival chain from p1 to p2 by du.
__device__ __forceinline__ void chain_step(const PointState& p1, PointState& p2, float du,
                                           float& comp) {
    const float y = du - comp;
    float t = p1.r + y;
    comp = (t - p1.r) - y;
    t = fminf(fmaxf(t, -4.0e8f), 4.0e8f);
    const float k = rintf(t);
    p2.r = t - k;
    p2.ki = p1.ki + (int)k;
}

// Bin decision from (ki, r); falls back to the reference's exact FP64
// evaluation when r is within `band` of +-1/2.
__device__ __forceinline__ bool decide(PointState& S, float band, const double4_32a* tx,
                                       int64_t i, const PixelCtx& px, const Anchor& A) {
    const float d = 0.5f - fabsf(S.r);  // distance to the nearest half-integer
    if (d <= band) {
        const double ts = exact_retarded_time(tx[i], px.P);
        S.idx = exact_bin(ts, px.w);
        S.flags = exact_flags(ts, px.w);
        // continue from the exact value
        double v = (ts - px.w.t0) * px.inv_dt - (double)A.B;
        v = fmax(-kBinLimit, fmin(v, kBinLimit));
        const double k = floor(v + 0.5);
        S.ki = (int)k;
        S.r = (float)(v - k);
        return true;
    }
    int k = A.Bi + S.ki;
    const int nt = px.w.nt;
    k = k < -2 ? -2 : (k > nt + 1 ? nt + 1 : k);
    S.idx = k;
    S.flags = (k < 0 ? kLeTmin : 0) | (k < nt ? kLtTmax : 0);
    return false;
}

// Start a compensated arrival chain at an anchor point.
__device__ __forceinline__ void start_chain(PointState& S, const Anchor& A) {
    const float k = rintf(A.frac);  // 0 or 1
    S.ki = (int)k;
    S.r = A.frac - k;
}

// Re-express a point against a new anchor.
__device__ __forceinline__ void rebase(PointState& S, const Anchor& from, const Anchor& to) {
    S.ki += (int)(from.B - to.B);
}

// ---------------------------------------------------------------------------
// The deposit of one step in bin units from (ki, r) coordinates on base Bi;
// the same branch structure and weights as deposit_step (lw_common.cuh),
// src/particle.cpp:786-865.
// ---------------------------------------------------------------------------
template <class Sink>
__device__ __forceinline__ bool deposit_step32(const PointState& p1, const PointState& p2, int Bi,
                                               int nt, Sink& sink) {
    if ((p2.flags & kLeTmin) || !(p1.flags & kLtTmax)) return false;
    const float dts = (float)(p2.ki - p1.ki) + (p2.r - p1.r);
    float field[6];
    const int idx2 = p2.idx > nt ? nt : p2.idx;
    const int u1i = Bi + p1.ki, u2i = Bi + p2.ki;  // integer parts of u1, u2
    if (!(p1.flags & kLeTmin) && p1.idx == idx2) {
        // the common case: the step lies within one bin
        const float wb = 0.5f * dts;
#pragma unroll
        for (int c = 0; c < 6; c++) field[c] = (p1.f[c] + p2.f[c]) * wb;
        sink.add(idx2, field);
        return true;
    }
    const float rd = __fdividef(1.0f, dts);
    int kfull0;
    if (p1.flags & kLeTmin) {
        kfull0 = 0;
    } else {
        // first partial bin idx1
        const int idx1 = p1.idx;
        const float b2 = (float)(u2i - idx1) - 0.5f + p2.r;  // ts2 - t_end
        const float b1 = (float)(idx1 - u1i) + 0.5f - p1.r;  // t_end - ts1
        const float w1 = b2 * rd, w2 = b1 * rd, wb = 0.5f * b1;
#pragma unroll
        for (int c = 0; c < 6; c++) field[c] = (p1.f[c] * (1.0f + w1) + p2.f[c] * w2) * wb;
        sink.add(idx1, field);
        kfull0 = idx1 + 1;
    }
    for (int k = kfull0; k < idx2; k++) {
        const float w1 = ((float)(u2i - k) + p2.r) * rd;
        const float w2 = ((float)(k - u1i) - p1.r) * rd;
#pragma unroll
        for (int c = 0; c < 6; c++) field[c] = p1.f[c] * w1 + p2.f[c] * w2;
        sink.add(k, field);
    }
    if (idx2 < nt) {
        const float a2 = (float)(u2i - idx2) + p2.r + 0.5f;  // ts2 - t_start
        const float a1 = (float)(idx2 - u1i) - 0.5f - p1.r;  // t_start - ts1
        const float w1 = a2 * rd, w2 = a1 * rd, wb = 0.5f * a2;
#pragma unroll
        for (int c = 0; c < 6; c++) field[c] = (p1.f[c] * w1 + p2.f[c] * (w2 + 1.0f)) * wb;
        sink.add(idx2, field);
    }
    return true;
}

constexpr float kChainRel = 1.0e-6f;  // bound on the relative error of one FP32 increment

// ---------------------------------------------------------------------------
// Kernel 1 (block-uniform): all 256 pixels of a block walk the same steps of
// a particle (the union of their in-window ranges), with the trajectory
// streamed through shared memory in chunks of one segment (cp.async, double
// buffered) and read as broadcasts.  Best when neighbouring pixels see a
// particle's radiation at similar times (forward screens).
// ---------------------------------------------------------------------------
constexpr int kUThreads = 256;

struct __align__(16) ChunkBuf {
    float4 q0[kSegLen], q1[kSegLen], q2[kSegLen], q3[kSegLen];
};

__device__ __forceinline__ void stage_chunk(ChunkBuf* b, const DevTraj& tr, int64_t p0, int avail) {
    // thread t copies one float4: array t / kSegLen, point t % kSegLen
    const int t = threadIdx.x;
    const int arr = t / kSegLen, l = t % kSegLen;
    if (arr < 4 && l < avail) {
        const float4* src = arr == 0 ? tr.q0 : arr == 1 ? tr.q1 : arr == 2 ? tr.q2 : tr.q3;
        float4* dst = arr == 0 ? b->q0 : arr == 1 ? b->q1 : arr == 2 ? b->q2 : b->q3;
        const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + l);
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src + p0 + l)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__device__ __forceinline__ void wait_chunk_all_but_newest() {
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
}
__device__ __forceinline__ void wait_chunk_all() {
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

__global__ void __launch_bounds__(kUThreads, 2)
    lw_fp32_uniform_kernel(DevTraj tr, DevScreen sc, DevWork wk) {
    __shared__ ChunkBuf buf[2];
    __shared__ int red[2][kUThreads / 32];
    // the FP64 pixel constants are needed only at anchors and in the exact
    // fallback: kept in shared memory rather than in registers
    __shared__ PixelCtx pxs[kUThreads];
    const int slot = blockIdx.y;
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
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
        if (!active || last < first) {
            first = 0x7fffffff;
            last = -1;
        }
        // block-wide union of the ranges
        const int wf = warp_min(first), wl = warp_max(last);
        if (lane == 0) {
            red[0][warp] = wf;
            red[1][warp] = wl;
        }
        __syncthreads();
        int lo = red[0][0], hi = red[1][0];
#pragma unroll
        for (int k = 1; k < kUThreads / 32; k++) {
            lo = min(lo, red[0][k]);
            hi = max(hi, red[1][k]);
        }
        __syncthreads();  // red[] is rewritten for the next particle
        if (lo > hi) continue;
        const int start = lo & ~(kSegLen - 1);  // >= st_lo
        const int n_pts = hi + 2 - start;       // points start .. hi+1
        const int n_chunks = (n_pts + kSegLen - 1) >> kSegShift;
        const double4_32a* txp = tr.tx + po;
        stage_chunk(&buf[0], tr, po + start, min(kSegLen, npm - start));
        Anchor A;
        PointState p1, p2;
        float comp = 0.0f, chain_err = 0.0f;
        for (int c = 0; c < n_chunks; c++) {
            const int p0 = start + (c << kSegShift);
            if (c + 1 < n_chunks) {
                stage_chunk(&buf[(c + 1) & 1], tr, po + p0 + kSegLen,
                            min(kSegLen, npm - (p0 + kSegLen)));
                wait_chunk_all_but_newest();
            } else {
                wait_chunk_all();
            }
            __syncthreads();
            const ChunkBuf& B = buf[c & 1];
            // the segment's anchor
            {
                Anchor An;
                make_anchor(An, txp[p0], px);
                if (c > 0) rebase(p1, A, An);
                A = An;
            }
            const int n_here = min(kSegLen, n_pts - (c << kSegShift));
            for (int l = 0; l < n_here; l++) {
                const int i = p0 + l;
                point_field(p2, B.q0[l], B.q1[l], B.q2[l], A);
                if (l == 0) {
                    start_chain(p2, A);
                    comp = 0.0f;
                    chain_err = 0.0f;
                } else {
                    const float du = step_increment(p1, p2, B.q3[l - 1], px.kdt);
                    chain_step(p1, p2, du, comp);
                    chain_err += fabsf(du) * kChainRel + 1.0e-7f;
                }
                if (decide(p2, A.err + chain_err, txp, i, px, A)) nfb++;
                if (i > start && active) {
                    if (deposit_step32(p1, p2, A.Bi, sc.nt, sink)) inwin++;
                }
                p1 = p2;
            }
            __syncthreads();  // the buffer is restaged two chunks later
        }
    }
    sink.flush();
    if (sink.err) atomicOr(wk.status, sink.err);
    inwin = warp_sum_u64(active ? inwin : 0);
    nfb = warp_sum_u64(active ? nfb : 0);
    unsigned long long nadd = warp_sum_u64(sink.n_add);
    if (lane == 0 && wk.counters) {
        if (inwin) atomicAdd(wk.counters, inwin);
        if (nfb) atomicAdd(wk.counters + 1, nfb);
        if (nadd) atomicAdd(wk.counters + 2, nadd);
    }
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
        int start = first & ~(kSegLen - 1);
        if (start < st_lo) start = st_lo;
        const int trips = last >= first ? last - start + 1 : 0;
        const int max_trips = warp_max(trips);
        if (max_trips == 0) continue;
        if (trips == 0) start = st_lo;
        const double4_32a* txp = tr.tx + po;
        const float4 *q0 = tr.q0 + po, *q1 = tr.q1 + po, *q2 = tr.q2 + po, *q3 = tr.q3 + po;
        Anchor A;
        make_anchor(A, txp[start], px);
        PointState p1, p2;
        point_field(p1, __ldg(q0 + start), __ldg(q1 + start), __ldg(q2 + start), A);
        start_chain(p1, A);
        if (decide(p1, A.err, txp, start, px, A)) nfb++;
        float comp = 0.0f, chain_err = 0.0f;
        for (int j = 0; j < max_trips; ++j) {
            const int i2 = start + j + 1;
            const bool live = j < trips;
            const bool boundary = (i2 & (kSegLen - 1)) == 0;
            if (boundary) {  // uniform: every lane's start is a segment boundary
                const int i2c = i2 < npm ? i2 : ((npm - 1) & ~(kSegLen - 1));
                Anchor An;
                make_anchor(An, txp[i2c], px);
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
    if ((threadIdx.x & 31) == 0 && wk.counters) {
        if (inwin) atomicAdd(wk.counters, inwin);
        if (nfb) atomicAdd(wk.counters + 1, nfb);
        if (nadd) atomicAdd(wk.counters + 2, nadd);
    }
}

cudaError_t launch_fp32(const DevTraj& tr, const DevScreen& sc, const DevWork& w, int variant,
                        cudaStream_t s) {
    if (variant == kVariantLanes) {
        dim3 grid((sc.np + 127) / 128, w.n_slots);
        lw_fp32_lanes_kernel<<<grid, 128, 0, s>>>(tr, sc, w);
    } else {
        dim3 grid((sc.np + kUThreads - 1) / kUThreads, w.n_slots);
        lw_fp32_uniform_kernel<<<grid, kUThreads, 0, s>>>(tr, sc, w);
    }
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
            double u = (t - t0) / dt;
            u = fmax(-kBinLimit, fmin(u, kBinLimit));
            const double k = floor(u + 0.5);
            p2.ki = (int)k;
            p2.r = (float)(u - k);
            p2.idx = exact_bin(t, w);
            p2.flags = exact_flags(t, w);
            for (int c = 0; c < 6; c++) p2.f[c] = (float)f[6 * (o + s) + c];
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
// m walks its points as both kernels do (anchor, FP32 chain, decision).
// u_est is the estimate before any exact fallback, band the bound used.
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
    make_anchor(A, txp[start], px);
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
