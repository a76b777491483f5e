// lw_fp32_point.cuh -- device functions of the split-precision path shared by
// its kernels (lw_fp32_main.cu, lw_fp32_warp.cu): the per-pixel double-float
// constants, the FP64 segment anchors, the FP32 field of one trajectory point,
// the compensated FP32 arrival chain with its error bound, the exact-fallback
// decision and the deposit of one step in bin units.  The derivations are in
// the header comment of lw_fp32_main.cu.
#pragma once

#include <cuda_runtime.h>

#include "lw_common.cuh"

namespace teufel {

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
// Packed FP32 pairs: one add.f32x2 / mul.f32x2 / fma.f32x2 instruction does
// two IEEE round-to-nearest single-precision operations.
// ---------------------------------------------------------------------------
union F2U {
    float2 f;
    unsigned long long u;
};
__device__ __forceinline__ float2 splat2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    F2U x, y, r;
    x.f = a;
    y.f = b;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(x.u), "l"(y.u));
    return r.f;
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    F2U x, y, r;
    x.f = a;
    y.f = b;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(x.u), "l"(y.u));
    return r.f;
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    F2U x, y, r;
    x.f = a;
    y.f = b;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(x.u), "l"(y.u));
    return r.f;
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    F2U x, y, z, r;
    x.f = a;
    y.f = b;
    z.f = c;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.u) : "l"(x.u), "l"(y.u), "l"(z.u));
    return r.f;
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

// v <- R v in the set's frame (FP64)
__device__ __forceinline__ void to_frame(const Frame& F, double& x, double& y, double& z) {
    if (F.identity) return;
    const double a = fma(F.r[0], x, fma(F.r[1], y, F.r[2] * z));
    const double b = fma(F.r[3], x, fma(F.r[4], y, F.r[5] * z));
    const double c = fma(F.r[6], x, fma(F.r[7], y, F.r[8] * z));
    x = a;
    y = b;
    z = c;
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

// Anchor of a chain that starts at trajectory point a, with positions measured
// from point b (the first point of a's segment, to which the per-point
// offsets e are relative).
__device__ __forceinline__ void make_anchor(Anchor& A, const double4_32a a, const double4_32a b,
                                            const PixelCtx& px, const Frame& F) {
    const double dx = px.P.x - b.y, dy = px.P.y - b.z, dz = px.P.z - b.w;
    if (F.identity) {
        A.Dx = (float)dx;
        A.Dy = (float)dy;
        A.Dz = (float)dz;
    } else {
        // the distance vector in the set's frame, formed in FP64
        A.Dx = (float)fma(F.r[0], dx, fma(F.r[1], dy, F.r[2] * dz));
        A.Dy = (float)fma(F.r[3], dx, fma(F.r[4], dy, F.r[5] * dz));
        A.Dz = (float)fma(F.r[6], dx, fma(F.r[7], dy, F.r[8] * dz));
    }
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
    // our rounding (t, P^.x/c and their sum, G/c, the sum with Tp, the
    // scaling: (|t| + |P^.x|/c + |Tp| + G/c)/dt + |u|, times 4.5e-16), the
    // reference's rounding of t + R/c (|t|/dt times 4.5e-16) and of t0 and the
    // flight time (refb0), and 1e-7 for the FP32 remainder
    const double mag = fma(fabs(pa) + G, ic, 2.0 * fabs(a.x) + fabs(px.Tp));
    A.err = (float)(fma(mag, px.inv_dt, fabs(u)) * 4.5e-16) + (1.0e-7f + px.refb0);
    if (u != u0) A.err = 1.0f;  // clamped: resolve the segment exactly
}
__device__ __forceinline__ void make_anchor(Anchor& A, const double4_32a a, const PixelCtx& px,
                                            const Frame& F) {
    make_anchor(A, a, a, px, F);
}

struct PointState {
    int ki;        // integer part of (ts - t0)/dt - B
    float r;       // the rest
    int idx;       // bin index round((ts-t0)/dt), clamped to [-2, nt+1]
    int flags;     // kLeTmin | kLtTmax | kExact
    float dt;      // duration of the trajectory step that starts at this point
    float Nx, Ny, Nz;
    float iR;      // 1/|R|
    float2 f[3];   // (Ex, Ey), (Ez, c*Bx), (c*By, c*Bz): packed for the f32x2 pipe
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
    S.iR = iR;
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
    const float irk2 = iR * rk * rk;
    const float cacc = irk2 * rk;   // 1/(R kappa^3), times scale/c folded into beta'
    const float cvel = c.w * iR * cacc;
    // N x ((N - beta) x beta') = (N - beta)(N.beta') - beta' (N.(N - beta)) with
    // N.(N - beta) = kappa, so E = (N - beta) s1 - beta' s2
    const float nbp = Nx * c.x + Ny * c.y + Nz * c.z;
    const float su = fmaf(cacc, nbp, cvel);
    const float sb = irk2;  // cacc * kappa
    const float Ex = mbx * su - c.x * sb;
    const float Ey = mby * su - c.y * sb;
    const float Ez = mbz * su - c.z * sb;
    S.f[0] = make_float2(Ex, Ey);
    S.f[1] = make_float2(Ez, Ny * Ez - Nz * Ey);
    S.f[2] = make_float2(Nz * Ex - Nx * Ez, Nx * Ey - Ny * Ex);
}

// 1 - c^.N for unit vectors, without cancellation: |c^ x N|^2 / (1 + c^.N)
// when c^.N > 0, else directly.
__device__ __forceinline__ float one_minus_cn(float cx, float cy, float cz, float Nx, float Ny,
                                              float Nz) {
    const float wx = cy * Nz - cz * Ny, wy = cz * Nx - cx * Nz, wz = cx * Ny - cy * Nx;
    const float cn = cx * Nx + cy * Ny + cz * Nz;
    return cn > 0.0f ? __fdividef(wx * wx + wy * wy + wz * wz, 1.0f + cn) : 1.0f - cn;
}

// Arrival increment of the step from point 1 to point 2 [bins].  With R1, R2
// the distance vectors, N = R/|R| and the chord x2 - x1 = beta_c c dt along
// the unit vector c^:
//   |R1| - |R2| = (x2 - x1).(R1 + R2) / (|R1| + |R2|) = beta_c c dt (c^.m),
//   m = (R1 + R2) / (|R1| + |R2|),
// so the increment is dt (1 - |beta_c| + |beta_c| (1 - c^.m)), and since
// (|R1| + |R2|)(1 - c^.m) = |R1| (1 - c^.N1) + |R2| (1 - c^.N2),
//   1 - c^.m = w1 (1 - c^.N1) + w2 (1 - c^.N2),  w1,2 = |R1,2| / (|R1| + |R2|):
// a weighted sum of non-negative terms, exact to rounding for any step length
// and distance (a step that passes close to the observation point included).
__device__ __forceinline__ float step_increment(const PointState& p1, const PointState& p2,
                                                float4 chord, float kdt) {
    const float t = __fdividef(1.0f, p1.iR + p2.iR);
    const float a1 = one_minus_cn(chord.x, chord.y, chord.z, p1.Nx, p1.Ny, p1.Nz);
    const float a2 = one_minus_cn(chord.x, chord.y, chord.z, p2.Nx, p2.Ny, p2.Nz);
    const float one_m_cm = fmaf(p2.iR * t, a1, p1.iR * t * a2);
    const float kap = chord.w + (1.0f - chord.w) * one_m_cm;
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
// The FP32 partial-trace sink.  Contributions to the same bin are summed in
// registers; the read half of the bin's read-modify-write is issued when the
// bin is opened and consumed only when it is closed, several steps later, so
// its memory latency overlaps the work of those steps instead of stalling the
// warp at every bin change.  All arithmetic is on packed pairs.
// ---------------------------------------------------------------------------
struct PrefetchSink {
    float2 a[3];
    float2 o[3];  // the partial trace's previous content of the open bin
    int open;
    int nt;
    float* row;  // this pixel's partial trace, [nt][6]
    unsigned int err;
    unsigned long long n_add;
    __device__ void init(float* r, int n) {
        row = r;
        nt = n;
        open = -1;
        err = 0;
        n_add = 0;
    }
    __device__ __forceinline__ void add(int k, const float2* f) {
        if (k < 0 || k >= nt) {
            err |= 1u << TEUFEL_ERR_RANGE;
            return;
        }
        n_add++;
        if (k == open) {
#pragma unroll
            for (int c = 0; c < 3; c++) a[c] = add2(a[c], f[c]);
        } else {
            flush();
            open = k;
            const float2* p = reinterpret_cast<const float2*>(row + (int64_t)k * 6);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                o[c] = p[c];
                a[c] = f[c];
            }
        }
    }
    __device__ __forceinline__ void flush() {
        if (open < 0) return;
        float2* p = reinterpret_cast<float2*>(row + (int64_t)open * 6);
#pragma unroll
        for (int c = 0; c < 3; c++) p[c] = add2(o[c], a[c]);
        open = -1;
    }
};

// The same contract without the prefetch: a closed bin is added to the
// partial trace with fire-and-forget vector reductions (red.global.add on
// float2), which the L2 performs, so the thread neither holds the bin's old
// content in registers nor waits for it.  Each pixel row is written by one
// thread only; the reductions are used for their latency, not for atomicity.
struct RedSink {
    float2 a[3];
    int open;
    int nt;
    float* row;  // this pixel's partial trace, [nt][6]
    unsigned int err;
    unsigned int n_add;
    __device__ void init(float* r, int n) {
        row = r;
        nt = n;
        open = -1;
        err = 0;
        n_add = 0;
    }
    __device__ __forceinline__ void add(int k, const float2* f) {
        if (k < 0 || k >= nt) {
            err |= 1u << TEUFEL_ERR_RANGE;
            return;
        }
        n_add++;
        if (k == open) {
#pragma unroll
            for (int c = 0; c < 3; c++) a[c] = add2(a[c], f[c]);
        } else {
            flush();
            open = k;
#pragma unroll
            for (int c = 0; c < 3; c++) a[c] = f[c];
        }
    }
    __device__ __forceinline__ void flush() {
        if (open < 0) return;
        float2* p = reinterpret_cast<float2*>(row + (int64_t)open * 6);
#pragma unroll
        for (int c = 0; c < 3; c++) atomicAdd(p + c, a[c]);
        open = -1;
    }
    // A regular step: f1 goes to bin k, in [0, nt); when `split`, f2 goes to
    // bin k+1, also in [0, nt).  In a chain of regular steps bin k is
    // already open, so the common work is the register accumulation.
    __device__ __forceinline__ void add_fast(int k, bool split, const float2* f1,
                                             const float2* f2) {
        if (k != open) {
            flush();
            open = k;
#pragma unroll
            for (int c = 0; c < 3; c++) a[c] = make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int c = 0; c < 3; c++) a[c] = add2(a[c], f1[c]);
        if (split) {
            float2* p = reinterpret_cast<float2*>(row + (int64_t)k * 6);
#pragma unroll
            for (int c = 0; c < 3; c++) atomicAdd(p + c, a[c]);
            open = k + 1;
        }
#pragma unroll
        for (int c = 0; c < 3; c++) a[c] = split ? f2[c] : a[c];
        n_add += split ? 2u : 1u;
    }
};

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
    float2 field[3];
    const int idx2 = p2.idx > nt ? nt : p2.idx;
    const int u1i = Bi + p1.ki, u2i = Bi + p2.ki;  // integer parts of u1, u2
    const float rd = __fdividef(1.0f, dts);
    if (!(p1.flags & kLeTmin) && idx2 - p1.idx <= 1) {
        // The common case, without branches: the step lies in bin idx1 or
        // crosses its upper edge e = idx1 + 1/2 into idx2 = idx1 + 1.  With
        // e' = min(u2, e) and f(e') the interpolant there, bin idx1 receives
        // (e' - u1)(f1 + f(e'))/2 and bin idx2 (u2 - e')(f(e') + f2)/2 -- the
        // single-bin weight (f1 + f2)/2 dts, and the first and last partial
        // bins of the reference (src/particle.cpp:835-862), in one form.
        const bool split = idx2 > p1.idx;
        const float a = split ? (float)(p1.idx - u1i) + 0.5f - p1.r : dts;  // e' - u1
        const float2 lam = splat2(split ? a * rd : 1.0f);  // no 0/0 for a zero-length step
        float2 fe[3];
#pragma unroll
        for (int c = 0; c < 3; c++) fe[c] = fma2(sub2(p2.f[c], p1.f[c]), lam, p1.f[c]);
        const float2 w1 = splat2(0.5f * a);
#pragma unroll
        for (int c = 0; c < 3; c++) field[c] = mul2(add2(p1.f[c], fe[c]), w1);
        sink.add(p1.idx, field);
        if (split && idx2 < nt) {
            const float2 w2 = splat2(0.5f * (dts - a));
#pragma unroll
            for (int c = 0; c < 3; c++) field[c] = mul2(add2(fe[c], p2.f[c]), w2);
            sink.add(idx2, field);
        }
        return true;
    }
    int kfull0;
    if (p1.flags & kLeTmin) {
        kfull0 = 0;
    } else {
        // first partial bin idx1
        const int idx1 = p1.idx;
        const float b2 = (float)(u2i - idx1) - 0.5f + p2.r;  // ts2 - t_end
        const float b1 = (float)(idx1 - u1i) + 0.5f - p1.r;  // t_end - ts1
        const float2 w1 = splat2(1.0f + b2 * rd), w2 = splat2(b1 * rd), wb = splat2(0.5f * b1);
#pragma unroll
        for (int c = 0; c < 3; c++) field[c] = mul2(fma2(p1.f[c], w1, mul2(p2.f[c], w2)), wb);
        sink.add(idx1, field);
        kfull0 = idx1 + 1;
    }
    for (int k = kfull0; k < idx2; k++) {
        const float2 w1 = splat2(((float)(u2i - k) + p2.r) * rd);
        const float2 w2 = splat2(((float)(k - u1i) - p1.r) * rd);
#pragma unroll
        for (int c = 0; c < 3; c++) field[c] = fma2(p1.f[c], w1, mul2(p2.f[c], w2));
        sink.add(k, field);
    }
    if (idx2 < nt) {
        const float a2 = (float)(u2i - idx2) + p2.r + 0.5f;  // ts2 - t_start
        const float a1 = (float)(idx2 - u1i) - 0.5f - p1.r;  // t_start - ts1
        const float2 w1 = splat2(a2 * rd), w2 = splat2(1.0f + a1 * rd), wb = splat2(0.5f * a2);
#pragma unroll
        for (int c = 0; c < 3; c++) field[c] = mul2(fma2(p1.f[c], w1, mul2(p2.f[c], w2)), wb);
        sink.add(idx2, field);
    }
    return true;
}

// A regular step: both points resolved without the exact fallback, both bins
// inside the trace (0 <= B + ki < nt, which implies ts > tmin and ts < tmax
// since |r| stays below 1/2 by more than the error bound), and ki2 - ki1 in
// {0, 1}.  deposit_step32 then takes its common branch with idx1 = B + ki1 and
// a = 1/2 - r1; this is that branch without the flag and range logic.
template <class Sink>
__device__ __forceinline__ void deposit_fast(const PointState& p1, const PointState& p2, int Bi,
                                             Sink& sink) {
    const bool split = p2.ki != p1.ki;
    const float dts = (split ? 1.0f : 0.0f) + (p2.r - p1.r);
    const float a = split ? 0.5f - p1.r : dts;
    const float2 lam = splat2(split ? a * __fdividef(1.0f, dts) : 1.0f);
    float2 fe[3], field1[3], field2[3];
#pragma unroll
    for (int c = 0; c < 3; c++) fe[c] = fma2(sub2(p2.f[c], p1.f[c]), lam, p1.f[c]);
    const float2 w1 = splat2(0.5f * a), w2 = splat2(0.5f * (dts - a));
#pragma unroll
    for (int c = 0; c < 3; c++) {
        field1[c] = mul2(add2(p1.f[c], fe[c]), w1);
        field2[c] = mul2(add2(fe[c], p2.f[c]), w2);
    }
    sink.add_fast(Bi + p1.ki, split, field1, field2);
}

// Bin index and window flags of a point that was not resolved exactly, from
// its chain coordinates (an exactly resolved point keeps its own).
__device__ __forceinline__ void materialize(PointState& S, int Bi, int nt) {
    if (S.flags & kExact) return;
    int k = Bi + S.ki;
    k = k < -2 ? -2 : (k > nt + 1 ? nt + 1 : k);
    S.idx = k;
    S.flags = (k < 0 ? kLeTmin : 0) | (k < nt ? kLtTmax : 0);
}

// The exact FP64 evaluation of a point whose estimate lies within its error
// bound of a half-integer: the reference's bin index and window flags, and
// the chain continued from the exact value (relative to anchor base B).
// Kept out of line: it is rare, and its FP64 temporaries would otherwise
// crowd the registers of the loop around it.
struct ExactPoint {
    int ki;
    float r;
    int idx;
    int flags;
};
static __device__ __noinline__ ExactPoint exact_point(const double4_32a* tx, int64_t i,
                                               const PixelCtx& px, int B) {
    ExactPoint e;
    const double ts = exact_retarded_time(tx[i], px.P);
    e.idx = exact_bin(ts, px.w);
    e.flags = exact_flags(ts, px.w);
    double v = (ts - px.w.t0) * px.inv_dt - (double)B;
    v = fmax(-kBinLimit, fmin(v, kBinLimit));
    const double k = floor(v + 0.5);
    e.ki = (int)k;
    e.r = (float)(v - k);
    return e;
}
__device__ __forceinline__ void apply_exact(PointState& S, const ExactPoint& e) {
    S.ki = e.ki;
    S.r = e.r;
    S.idx = e.idx;
    S.flags = e.flags;
}

// Bin decision from (ki, r); falls back to the reference's exact FP64
// evaluation when r is within `band` of +-1/2.  Returns true on a fallback.
__device__ __forceinline__ bool decide(PointState& S, float band, const double4_32a* tx,
                                       int64_t i, const PixelCtx& px, const Anchor& A) {
    if (0.5f - fabsf(S.r) <= band) {
        apply_exact(S, exact_point(tx, i, px, A.Bi));
        return true;
    }
    S.flags = 0;
    materialize(S, A.Bi, px.w.nt);
    return false;
}

constexpr float kChainRel = 1.0e-6f;  // bound on the relative error of one FP32 increment

// A chain is re-anchored in FP64 at the next chunk boundary once the error
// bound of any lane of the warp exceeds kReanchorBound [bins]: the rounding
// of the increments accumulates as a random walk (about 3e-7 |du| per step
// when the transverse direction components are ~1e-2 and the angles ~1e-3),
// so chains that advance by many bins per step are kept short, while chains
// that advance slowly run to the end of their segment.
constexpr float kReanchorBound = 2.7e-5f;
__device__ __forceinline__ bool warp_any_above(float v, float limit) {
    // non-negative floats order like their bit patterns
    return __reduce_max_sync(0xffffffffu, __float_as_uint(v)) > __float_as_uint(limit);
}

}  // namespace teufel
