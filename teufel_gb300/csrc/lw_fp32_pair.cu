// lw_fp32_pair.cu -- the split-precision kernel with two particles per
// thread.
//
// As the warp-uniform kernel (lw_fp32_warp.cu), each warp owns 32 pixels and
// walks trajectory points together, staged in shared memory.  Here every lane
// carries two particles (a pair, 2j and 2j+1) for its pixel, and all the
// per-point FP32 arithmetic -- the field, the arrival increment, the
// compensated chain and the deposit weights -- is done on packed pairs
// (add/sub/mul/fma.rn.f32x2), one instruction for both particles.  The
// trajectory data of a pair is interleaved component by component when the
// set is uploaded, so every operand pair comes straight out of shared memory.
// Bin decisions, fallbacks and the sink stay per particle.
//
// Both particles deposit into the lane's one pixel row; each keeps its own
// open bin.  A bin that both happen to hold open is added to twice by the
// fire-and-forget reductions, which is the sum the trace needs.
#include <cuda_runtime.h>

#include "lw_fp32_point.cuh"

namespace teufel {

// ---------------------------------------------------------------------------
// Preparation: the interleaved per-point data of every pair.
// ---------------------------------------------------------------------------
// A pair-point is kPairPoint float4, the two particles interleaved component
// by component (lo/hi halves: particle a, b):
//   0-1  e (offset from the segment's first point), dt of the step it starts
//   2-3  beta^, 1 - |beta|
//   4-5  scaled beta', velocity-field scale
//   6-7  dA = beta^_i - c^_i, 1 - |beta_c|   (c^_i: chord of the step i -> i+1)
//   8-9  dB = beta^_(i+1) - c^_i, unused
// all in the set's frame.  dA and dB give the arrival-increment shares
// 1 - c^.N = (1 - beta^.N) + d.N of the step's two end points from the field's
// own 1 - beta^.N; they are formed in FP64, so their FP32 values carry full
// relative precision however small they are.
// dA, dB of point k of a particle with points [o, o + n), in the set's frame
__device__ __forceinline__ void chord_offsets(const DevTraj& tr, int64_t o, int64_t n, int64_t k,
                                              double3& dA, double3& dB) {
    auto bhat = [&](int64_t q) {
        const double4_32a bg = tr.pp[q];
        const double P = sqrt(bg.x * bg.x + bg.y * bg.y + bg.z * bg.z);
        return P > 0.0 ? make_double3(bg.x / P, bg.y / P, bg.z / P) : make_double3(0.0, 0.0, 1.0);
    };
    double3 c = make_double3(0.0, 0.0, 1.0);
    const double3 b1 = bhat(k);
    double3 b2 = b1;
    if (k + 1 < o + n) {
        const double4_32a p = tr.tx[k], q = tr.tx[k + 1];
        const double ex = q.y - p.y, ey = q.z - p.z, ez = q.w - p.w;
        const double L = sqrt(ex * ex + ey * ey + ez * ez);
        if (L > 0.0) c = make_double3(ex / L, ey / L, ez / L);
        b2 = bhat(k + 1);
    } else {
        c = b1;  // no step starts at the last point
    }
    dA = make_double3(b1.x - c.x, b1.y - c.y, b1.z - c.z);
    dB = make_double3(b2.x - c.x, b2.y - c.y, b2.z - c.z);
    to_frame(tr.frame, dA.x, dA.y, dA.z);
    to_frame(tr.frame, dB.x, dB.y, dB.z);
}

__global__ void prep_pairs_kernel(DevTraj tr, float4* pq) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = tr.pair_offsets[tr.n_pairs];
    if (i >= total) return;
    int lo = 0, hi = tr.n_pairs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (tr.pair_offsets[mid] <= i) lo = mid; else hi = mid - 1;
    }
    const int j = lo;
    const int64_t l = i - tr.pair_offsets[j];
    const int ma = 2 * j, mb = 2 * j + 1 < tr.n_particles ? 2 * j + 1 : 2 * j;
    const int64_t oa = tr.offsets[ma], na = tr.offsets[ma + 1] - oa;
    const int64_t ob = tr.offsets[mb], nb = tr.offsets[mb + 1] - ob;
    float4 a0, a1, a2, a3, b0, b1, b2, b3;
    double3 dAa = make_double3(0.0, 0.0, 0.0), dBa = dAa, dAb = dAa, dBb = dAa;
    if (na > 0) {
        const int64_t k = oa + (l < na ? l : na - 1);
        a0 = tr.q0[k]; a1 = tr.q1[k]; a2 = tr.q2[k]; a3 = tr.q3[k];
        chord_offsets(tr, oa, na, k, dAa, dBa);
    } else {
        a0 = a1 = a2 = a3 = make_float4(0.0f, 0.0f, 1.0f, 1.0f);
    }
    if (nb > 0) {
        const int64_t k = ob + (l < nb ? l : nb - 1);
        b0 = tr.q0[k]; b1 = tr.q1[k]; b2 = tr.q2[k]; b3 = tr.q3[k];
        chord_offsets(tr, ob, nb, k, dAb, dBb);
    } else {
        b0 = a0; b1 = a1; b2 = a2; b3 = a3;
        dAb = dAa;
        dBb = dBa;
    }
    float4* o = pq + kPairPoint * i;
    o[0] = make_float4(a0.x, b0.x, a0.y, b0.y);
    o[1] = make_float4(a0.z, b0.z, a0.w, b0.w);
    o[2] = make_float4(a1.x, b1.x, a1.y, b1.y);
    o[3] = make_float4(a1.z, b1.z, a1.w, b1.w);
    o[4] = make_float4(a2.x, b2.x, a2.y, b2.y);
    o[5] = make_float4(a2.z, b2.z, a2.w, b2.w);
    o[6] = make_float4((float)dAa.x, (float)dAb.x, (float)dAa.y, (float)dAb.y);
    o[7] = make_float4((float)dAa.z, (float)dAb.z, a3.w, b3.w);
    o[8] = make_float4((float)dBa.x, (float)dBb.x, (float)dBa.y, (float)dBb.y);
    o[9] = make_float4((float)dBa.z, (float)dBb.z, 0.0f, 0.0f);
}

cudaError_t launch_prep_pairs(const DevTraj& tr, cudaStream_t s) {
    if (tr.n_pairs <= 0) return cudaSuccess;
    // the pair-point count is read on the device; launch for an upper bound
    const int64_t bound = tr.n_points;  // >= sum over pairs of max(na, nb)
    prep_pairs_kernel<<<(unsigned)((bound + 255) / 256), 256, 0, s>>>(tr,
                                                                     const_cast<float4*>(tr.pq));
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Packed pairs: .x is particle a, .y particle b.
// ---------------------------------------------------------------------------
struct F2 {
    float2 v;
};
__device__ __forceinline__ F2 f2(float a, float b) { return F2{make_float2(a, b)}; }
__device__ __forceinline__ F2 f2(float2 a) { return F2{a}; }
__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return F2{add2(a.v, b.v)}; }
__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return F2{sub2(a.v, b.v)}; }
__device__ __forceinline__ F2 operator*(F2 a, F2 b) { return F2{mul2(a.v, b.v)}; }
__device__ __forceinline__ F2 fma(F2 a, F2 b, F2 c) { return F2{fma2(a.v, b.v, c.v)}; }
__device__ __forceinline__ F2 rsqrt2(F2 a) { return f2(rsqrtf(a.v.x), rsqrtf(a.v.y)); }
__device__ __forceinline__ F2 rcp2(F2 a) {
    return f2(__fdividef(1.0f, a.v.x), __fdividef(1.0f, a.v.y));
}
struct V2 {
    F2 x, y, z;
};
__device__ __forceinline__ V2 cross(const V2& a, const V2& b) {
    return V2{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ F2 dot(const V2& a, const V2& b) {
    return fma(a.x, b.x, fma(a.y, b.y, a.z * b.z));
}
__device__ __forceinline__ V2 operator+(const V2& a, const V2& b) {
    return V2{a.x + b.x, a.y + b.y, a.z + b.z};
}
__device__ __forceinline__ V2 operator-(const V2& a, const V2& b) {
    return V2{a.x - b.x, a.y - b.y, a.z - b.z};
}
__device__ __forceinline__ V2 operator*(const V2& a, F2 s) { return V2{a.x * s, a.y * s, a.z * s}; }

// The kPairPoint float4 of one pair-point, as staged in shared memory.
struct PairPoint {
    float4 d[kPairPoint];
};
__device__ __forceinline__ F2 lo2(float4 v) { return f2(v.x, v.y); }
__device__ __forceinline__ F2 hi2(float4 v) { return f2(v.z, v.w); }

struct PointState2 {
    int ka, kb;     // ki of particles a, b
    F2 r;
    int idxa, idxb; // bin indices (general path only)
    int fla, flb;   // window flags; kExact when resolved exactly, else 0 until materialized
    bool rega, regb;  // resolved without fallback, bin inside the trace
    F2 iR;          // 1/|R|
    F2 aplus;       // 1 - c^.N with c^ the chord of the step this point starts
    F2 f[6];        // Ex, Ey, Ez, cBx, cBy, cBz
};

// The anchors of both particles, as the loop uses them.
struct Anchor2 {
    V2 D;
    F2 err;
    F2 frac;
    int Ba, Bb;
};
__device__ __forceinline__ Anchor2 pack_anchor(const Anchor& a, const Anchor& b) {
    Anchor2 A;
    A.D = V2{f2(a.Dx, b.Dx), f2(a.Dy, b.Dy), f2(a.Dz, b.Dz)};
    A.err = f2(a.err, b.err);
    A.frac = f2(a.frac, b.frac);
    A.Ba = a.Bi;
    A.Bb = b.Bi;
    return A;
}

// point_field (lw_fp32_point.cuh) for both particles at once, plus the point's
// shares of the arrival increments (step_increment2): 1 - c^.N for the chord
// of the step that ends here (from qprev's dB, returned in aminus) and of the
// step that starts here (from q's dA, kept in S.aplus), as 1 - beta^.N + d.N.
__device__ __forceinline__ void point_field2(PointState2& S, const PairPoint& q,
                                             const PairPoint& qprev, const Anchor2& A,
                                             F2& aminus) {
    const V2 e{lo2(q.d[0]), hi2(q.d[0]), lo2(q.d[1])};
    const V2 b{lo2(q.d[2]), hi2(q.d[2]), lo2(q.d[3])};
    const F2 eps = hi2(q.d[3]);
    const V2 c{lo2(q.d[4]), hi2(q.d[4]), lo2(q.d[5])};
    const F2 cw = hi2(q.d[5]);
    const F2 one = f2(1.0f, 1.0f);
    const V2 D = A.D - e;
    const F2 iR = rsqrt2(dot(D, D));
    const V2 N = D * iR;
    S.iR = iR;
    const V2 W = cross(b, N);
    const F2 rc1 = rcp2(one + dot(b, N));
    const F2 a0 = dot(W, W) * rc1;  // 1 - beta^.N
    const F2 kappa = fma(one - eps, a0, eps);
    S.aplus = a0 + dot(V2{lo2(q.d[6]), hi2(q.d[6]), lo2(q.d[7])}, N);
    aminus = a0 + dot(V2{lo2(qprev.d[8]), hi2(qprev.d[8]), lo2(qprev.d[9])}, N);
    const V2 Sv = N + b;
    const V2 T = cross(W, Sv);
    const V2 mb{fma(T.x, rc1, b.x * eps), fma(T.y, rc1, b.y * eps), fma(T.z, rc1, b.z * eps)};
    const F2 rk = rcp2(kappa);
    const F2 irk2 = iR * rk * rk;
    const F2 cacc = irk2 * rk;
    const F2 su = fma(cacc, dot(N, c), cw * iR * cacc);
    const V2 E = mb * su - c * irk2;
    const V2 Bv = cross(N, E);
    S.f[0] = E.x;
    S.f[1] = E.y;
    S.f[2] = E.z;
    S.f[3] = Bv.x;
    S.f[4] = Bv.y;
    S.f[5] = Bv.z;
}

// The arrival increment of the step from point 1 to point 2 [bins] for both
// particles: step_increment (lw_fp32_point.cuh) with the points' shares
// 1 - c^.N formed when each point was evaluated (point_field2), so a point
// state carries two numbers instead of N.  q is the pair-point the step
// starts at (its chord and dt).
__device__ __forceinline__ F2 step_increment2(const PointState2& p1, const PointState2& p2,
                                              F2 aminus, const PairPoint& q, F2 kdt) {
    const F2 ceps = hi2(q.d[7]);
    const F2 dt = hi2(q.d[1]);
    const F2 t = rcp2(p1.iR + p2.iR);
    const F2 one_m_cm = fma(p2.iR * t, p1.aplus, p1.iR * t * aminus);
    const F2 kap = fma(f2(1.0f, 1.0f) - ceps, one_m_cm, ceps);
    return dt * kdt * kap;
}

__device__ __forceinline__ void chain_step2(const PointState2& p1, PointState2& p2, F2 du,
                                            F2& comp) {
    const F2 y = du - comp;
    F2 t = p1.r + y;
    comp = (t - p1.r) - y;
    const float tx = fminf(fmaxf(t.v.x, -4.0e8f), 4.0e8f);
    const float ty = fminf(fmaxf(t.v.y, -4.0e8f), 4.0e8f);
    const float kx = rintf(tx), ky = rintf(ty);
    p2.r = f2(tx, ty) - f2(kx, ky);
    p2.ka = p1.ka + (int)kx;
    p2.kb = p1.kb + (int)ky;
}

__device__ __forceinline__ void start_chain2(PointState2& S, const Anchor2& A) {
    const float kx = rintf(A.frac.v.x), ky = rintf(A.frac.v.y);
    S.ka = (int)kx;
    S.kb = (int)ky;
    S.r = A.frac - f2(kx, ky);
}

// One particle of a pair as a PointState, for the general deposit.
template <int W>
__device__ __forceinline__ PointState unpack(const PointState2& S) {
    PointState p;
    p.ki = W ? S.kb : S.ka;
    p.r = W ? S.r.v.y : S.r.v.x;
    p.idx = W ? S.idxb : S.idxa;
    p.flags = W ? S.flb : S.fla;
#pragma unroll
    for (int c = 0; c < 3; c++)
        p.f[c] = W ? make_float2(S.f[2 * c].v.y, S.f[2 * c + 1].v.y)
                   : make_float2(S.f[2 * c].v.x, S.f[2 * c + 1].v.x);
    return p;
}

// The six components of one bin, added by three red.global.add.v2.f32 under
// one predicate: the L2 adds them when p holds.  One asm block, so the
// predicate is formed once and the addresses are immediate offsets.
__device__ __forceinline__ void red_add6_if(bool p, float* addr, float a0, float a1, float a2,
                                            float a3, float a4, float a5) {
    asm volatile(
        "{\n\t.reg .pred q;\n\tsetp.ne.b32 q, %0, 0;\n\t"
        "@q red.global.add.v2.f32 [%1], {%2, %3};\n\t"
        "@q red.global.add.v2.f32 [%1+8], {%4, %5};\n\t"
        "@q red.global.add.v2.f32 [%1+16], {%6, %7};\n\t}"
        ::"r"((int)p), "l"(addr), "f"(a0), "f"(a1), "f"(a2), "f"(a3), "f"(a4), "f"(a5)
        : "memory");
}

// ---------------------------------------------------------------------------
// The sink of a lane: one pixel row, an open bin per particle, accumulators
// in packed form (component c of particles a and b).  Closed bins are added
// with fire-and-forget reductions, as RedSink (lw_fp32_point.cuh) does.
// ---------------------------------------------------------------------------
struct PairSink {
    F2 acc[6];
    int open_a, open_b;
    float* row;
    unsigned int err;
    unsigned int n_add;
    __device__ void init(float* r) {
        row = r;
        open_a = open_b = -1;
        err = 0;
        n_add = 0;
#pragma unroll
        for (int c = 0; c < 6; c++) acc[c] = f2(0.0f, 0.0f);
    }
    template <int W>
    __device__ __forceinline__ float get(int c) const {
        return W ? acc[c].v.y : acc[c].v.x;
    }
    template <int W>
    __device__ __forceinline__ void set(int c, float v) {
        if (W) acc[c].v.y = v; else acc[c].v.x = v;
    }
    template <int W>
    __device__ __forceinline__ void reduce_to(int k) {
        float2* p = reinterpret_cast<float2*>(row + (int64_t)k * 6);
        atomicAdd(p, make_float2(get<W>(0), get<W>(1)));
        atomicAdd(p + 1, make_float2(get<W>(2), get<W>(3)));
        atomicAdd(p + 2, make_float2(get<W>(4), get<W>(5)));
    }
    template <int W>
    __device__ __forceinline__ void flush() {
        int& open = W ? open_b : open_a;
        if (open < 0) return;
        reduce_to<W>(open);
        open = -1;
    }
    // The RedSink contract for particle W: f = component pairs (Ex,Ey),
    // (Ez,cBx), (cBy,cBz).
    template <int W>
    __device__ __forceinline__ void add(int k, const float2* f, int nt) {
        if (k < 0 || k >= nt) {
            err |= 1u << TEUFEL_ERR_RANGE;
            return;
        }
        n_add++;
        int& open = W ? open_b : open_a;
        if (k == open) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                set<W>(2 * c, get<W>(2 * c) + f[c].x);
                set<W>(2 * c + 1, get<W>(2 * c + 1) + f[c].y);
            }
        } else {
            flush<W>();
            open = k;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                set<W>(2 * c, f[c].x);
                set<W>(2 * c + 1, f[c].y);
            }
        }
    }
    // Regular steps of both particles: fa/fb say which particle deposits
    // (its weights are zero otherwise), ka/kb its bin, sa/sb whether the step
    // crosses into bin k+1.  Bin k receives f1 a1 + f2 b1, bin k+1 (on a
    // crossing) f1 a2 + f2 b2, fused into the accumulators.
    __device__ __forceinline__ void add_fast(bool fa, bool fb, int ka, int kb, bool sa, bool sb,
                                             const F2* f1, const F2* f2v, F2 a1, F2 b1, F2 a2,
                                             F2 b2) {
        // a bin other than the open one: only after a general-path step or at
        // the start of a walk, so one branch for both particles
        const bool na = fa && ka != open_a, nb = fb && kb != open_b;
        if (na || nb) {
            if (na) {
                flush<0>();
                open_a = ka;
#pragma unroll
                for (int c = 0; c < 6; c++) acc[c].v.x = 0.0f;
            }
            if (nb) {
                flush<1>();
                open_b = kb;
#pragma unroll
                for (int c = 0; c < 6; c++) acc[c].v.y = 0.0f;
            }
        }
#pragma unroll
        for (int c = 0; c < 6; c++) acc[c] = fma(f2v[c], b1, fma(f1[c], a1, acc[c]));
        // a step that crosses into the next bin closes its bin: predicated
        // reductions, no divergent branch
        reduce_if<0>(sa, ka);
        reduce_if<1>(sb, kb);
        open_a = sa ? ka + 1 : open_a;
        open_b = sb ? kb + 1 : open_b;
        const F2 keep = f2(sa ? 0.0f : 1.0f, sb ? 0.0f : 1.0f);
#pragma unroll
        for (int c = 0; c < 6; c++) acc[c] = fma(acc[c], keep, fma(f2v[c], b2, f1[c] * a2));
        n_add += (unsigned)fa + (unsigned)fb + (unsigned)sa + (unsigned)sb;
    }
    // Regular steps of both particles that may span several bins: ka/kb the
    // first bin, spa/spb >= 0 the bins spanned beyond it (0 for a particle
    // that does not deposit).  The first bin receives f1 a1 + f2 b1 and closes
    // when the step spans; each full bin k1 + j, 0 < j < span, receives
    // f1 w1(j) + f2 w2(j) with w1(j) = (u2 - j) rd, w2(j) = (j - u1) rd in bin
    // units from k1 (u1 = r1, u2 = span + r2); the last bin opens with
    // f1 a2 + f2 b2.
    __device__ __forceinline__ void add_multi(bool fa, bool fb, int ka, int kb, int spa, int spb,
                                              const F2* f1, const F2* f2v, F2 a1, F2 b1, F2 a2,
                                              F2 b2, F2 u1, F2 u2, F2 rd) {
        const bool na = fa && ka != open_a, nb = fb && kb != open_b;
        if (na || nb) {
            if (na) {
                flush<0>();
                open_a = ka;
#pragma unroll
                for (int c = 0; c < 6; c++) acc[c].v.x = 0.0f;
            }
            if (nb) {
                flush<1>();
                open_b = kb;
#pragma unroll
                for (int c = 0; c < 6; c++) acc[c].v.y = 0.0f;
            }
        }
#pragma unroll
        for (int c = 0; c < 6; c++) acc[c] = fma(f2v[c], b1, fma(f1[c], a1, acc[c]));
        const bool sa = spa > 0, sb = spb > 0;
        reduce_if<0>(sa, ka);
        reduce_if<1>(sb, kb);
        // full bins, in bin order per particle
        const int nfull = max(spa, spb) - 1;
        for (int j = 1; j <= nfull; j++) {
            const F2 jj = f2((float)j, (float)j);
            const F2 w1 = (u2 - jj) * rd, w2 = (jj - u1) * rd;
            F2 g[6];
#pragma unroll
            for (int c = 0; c < 6; c++) g[c] = fma(f2v[c], w2, f1[c] * w1);
            const bool pa = j < spa, pb = j < spb;
            float* qa = row + (int64_t)(ka + j) * 6;
            float* qb = row + (int64_t)(kb + j) * 6;
            red_add6_if(pa, qa, g[0].v.x, g[1].v.x, g[2].v.x, g[3].v.x, g[4].v.x, g[5].v.x);
            red_add6_if(pb, qb, g[0].v.y, g[1].v.y, g[2].v.y, g[3].v.y, g[4].v.y, g[5].v.y);
        }
        open_a = sa ? ka + spa : open_a;
        open_b = sb ? kb + spb : open_b;
        const F2 keep = f2(sa ? 0.0f : 1.0f, sb ? 0.0f : 1.0f);
#pragma unroll
        for (int c = 0; c < 6; c++) acc[c] = fma(acc[c], keep, fma(f2v[c], b2, f1[c] * a2));
        n_add += (unsigned)fa + (unsigned)fb + (unsigned)spa + (unsigned)spb;
    }
    template <int W>
    __device__ __forceinline__ void reduce_if(bool p, int k) {
        red_add6_if(p, row + (int64_t)k * 6, get<W>(0), get<W>(1), get<W>(2), get<W>(3),
                    get<W>(4), get<W>(5));
    }
};

// The decision taken for point i of particle m (particle W of the pair) at
// this lane's pixel: the exact evaluation's bin and flags where the point
// fell back to it, else the bin B + ki and the window flags it implies (as
// materialize does), into the decision record.  A point evaluated twice (the
// last point of one slot is the first of the next) must get the same
// decision both times; a difference is flagged.
template <int W>
__device__ __forceinline__ void record_point(const DevWork& wk, int n_particles, int pix, int m,
                                             int i, const PointState2& q, int B, int nt) {
    const int f = W ? q.flb : q.fla;
    int idx, fl;
    if (f & kExact) {
        idx = W ? q.idxb : q.idxa;
        fl = f;
    } else {
        int k = B + (W ? q.kb : q.ka);
        k = k < -2 ? -2 : (k > nt + 1 ? nt + 1 : k);
        idx = k;
        fl = (k < 0 ? kLeTmin : 0) | (k < nt ? kLtTmax : 0);
    }
    const int v = rec_encode(idx, fl);
    int* p = wk.rec + ((int64_t)pix * n_particles + m) * wk.rec_stride + i;
    const int old = atomicCAS(p, 0, v);
    if (old != 0 && old != v) atomicOr(p, kRecConflict);
}

template <int W>
struct PairView {
    PairSink* s;
    int nt;
    __device__ __forceinline__ void add(int k, const float2* f) { s->add<W>(k, f, nt); }
};

// Regular steps of both particles (deposit_fast, lw_fp32_point.cuh, in packed
// form).  fa/fb: the particle deposits a regular step.  The step's trapezoid
// (fields f1, f2 at arrival r1 < r2 [bins]) is split at the bin edge when it
// crosses one: with dts = r2 - r1 (+1 on a crossing), a the part in bin k
// (dts when no crossing), lam = a/dts and fe = (1 - lam) f1 + lam f2,
//   bin k:   (f1 + fe) a/2       = f1 (2 - lam) a/2       + f2 lam a/2,
//   bin k+1: (fe + f2) (dts-a)/2 = f1 (1 - lam) (dts-a)/2 + f2 (1 + lam) (dts-a)/2.
__device__ __forceinline__ void deposit_fast2(const PointState2& p1, const PointState2& p2,
                                              int Ba, int Bb, bool fa, bool fb, PairSink& sink) {
    const bool sa = fa && p2.ka != p1.ka, sb = fb && p2.kb != p1.kb;
    const F2 dts = f2(sa ? 1.0f : 0.0f, sb ? 1.0f : 0.0f) + (p2.r - p1.r);
    const F2 h = f2(0.5f, 0.5f) - p1.r;
    const F2 a = f2(sa ? h.v.x : dts.v.x, sb ? h.v.y : dts.v.y);
    // lam = 1 without a crossing: dts may be zero there (a particle past its
    // last point repeats it)
    const F2 q = a * rcp2(dts);
    const F2 lam = f2(sa ? q.v.x : 1.0f, sb ? q.v.y : 1.0f);
    const F2 hw1 = f2(fa ? 0.5f * a.v.x : 0.0f, fb ? 0.5f * a.v.y : 0.0f);
    const F2 hw2 = f2(0.5f, 0.5f) * (dts - a);  // zero without a crossing
    const F2 one = f2(1.0f, 1.0f);
    const F2 a1 = (f2(2.0f, 2.0f) - lam) * hw1, b1 = lam * hw1;
    const F2 a2 = (one - lam) * hw2, b2 = (one + lam) * hw2;
    sink.add_fast(fa, fb, Ba + p1.ka, Bb + p1.kb, sa, sb, p1.f, p2.f, a1, b1, a2, b2);
}

// Regular steps that span several bins (deposit_step32's first partial, full
// and last partial bins, for both particles at once).  A step that does not
// span (sp = 0) deposits its single-bin weight dts (f1 + f2)/2; a particle that
// does not deposit gets zero weights and no span.
constexpr int kMaxSpan = 16;  // bins a step of this path may span beyond its first

__device__ __forceinline__ void multi_weights(bool f, int sp, float r1, float r2, float& a1,
                                              float& b1, float& a2, float& b2, float& u2,
                                              float& rd) {
    const float dts = (float)sp + (r2 - r1);
    rd = __fdividef(1.0f, dts);
    u2 = (float)sp + r2;
    // first bin: from u1 to its upper edge; last bin: from its lower edge to u2
    const float h1 = 0.5f - r1, h2 = (float)sp - 0.5f + r2;
    const float g2 = r2 + 0.5f, g1 = (float)sp - 0.5f - r1;
    const float s1a = (1.0f + h2 * rd) * 0.5f * h1, s1b = h1 * rd * 0.5f * h1;
    const float s2a = g2 * rd * 0.5f * g2, s2b = (1.0f + g1 * rd) * 0.5f * g2;
    const bool spans = sp > 0;
    a1 = !f ? 0.0f : spans ? s1a : 0.5f * dts;
    b1 = !f ? 0.0f : spans ? s1b : 0.5f * dts;
    a2 = f && spans ? s2a : 0.0f;
    b2 = f && spans ? s2b : 0.0f;
}

__device__ __forceinline__ void deposit_multi2(const PointState2& p1, const PointState2& p2,
                                               int Ba, int Bb, bool fa, bool fb, PairSink& sink) {
    const int spa = fa ? p2.ka - p1.ka : 0, spb = fb ? p2.kb - p1.kb : 0;
    float a1x, b1x, a2x, b2x, u2x, rdx, a1y, b1y, a2y, b2y, u2y, rdy;
    multi_weights(fa, spa, p1.r.v.x, p2.r.v.x, a1x, b1x, a2x, b2x, u2x, rdx);
    multi_weights(fb, spb, p1.r.v.y, p2.r.v.y, a1y, b1y, a2y, b2y, u2y, rdy);
    sink.add_multi(fa, fb, Ba + p1.ka, Bb + p1.kb, spa, spb, p1.f, p2.f, f2(a1x, a1y), f2(b1x, b1y),
                   f2(a2x, a2y), f2(b2x, b2y), p1.r, f2(u2x, u2y), f2(rdx, rdy));
}

// ---------------------------------------------------------------------------
// The kernel
// ---------------------------------------------------------------------------
constexpr int kPThreads = kPairTile;  // one warp per block: residency is set by registers alone

// Chunks of 16 pair-points: two staged chunks and the lanes' pixel data stay
// within 10 KB per block, so 16 one-warp blocks fit an SM's shared memory.
// Anchors may move at chunk boundaries; segment boundaries stay chunk
// boundaries.
constexpr int kPChunkShift = 4;
constexpr int kPChunkLen = 1 << kPChunkShift;
static_assert(kSegLen % kPChunkLen == 0 && kPChunkLen % 2 == 0, "chunk layout");

// A staged chunk: p[0] is the pair-point before the chunk (the start of the
// chunk's first step), p[1 + l] the chunk's point l.
struct __align__(16) PairChunk {
    PairPoint p[kPChunkLen + 1];
};

// The 32 lanes copy pair-points p0-1 .. p0+avail-1 of the pair whose data
// starts at pq (p[0] only when p0 > 0).
__device__ __forceinline__ void pair_stage(PairChunk* b, const float4* pq, int p0, int avail,
                                           int lane) {
    const int skip = p0 > 0 ? 0 : kPairPoint;  // float4s of p[0] not copied
    const int n = kPairPoint * (avail + 1);
    const float4* src = pq + kPairPoint * ((int64_t)p0 - 1);
    float4* dst = reinterpret_cast<float4*>(b->p);
#pragma unroll
    for (int k = 0; k < (kPairPoint * (kPChunkLen + 1) + 31) / 32; k++) {
        const int t = lane + 32 * k;
        if (t >= skip && t < n) {
            const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + t);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src + t)
                         : "memory");
        }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

__device__ __forceinline__ int pair_of_segment(const int64_t* seg_offsets, int n, int64_t g) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (seg_offsets[mid + 1] > g) hi = mid; else lo = mid + 1;
    }
    return lo;
}

// In-window step range of particle m within local steps [st_lo, st_hi), or
// an empty range (first > last) when the lane has none.
__device__ __forceinline__ void particle_range(const DevTraj& tr, int m, int st_lo, int st_hi,
                                               bool active, const PixelCtx& px, int& first,
                                               int& last) {
    first = 0x7fffffff;
    last = -1;
    if (!active || st_lo >= st_hi) return;
    first = st_lo;
    last = st_hi - 1;
    if (tr.vhat[m].w > 0.0)
        inwindow_steps(tr.tx + tr.offsets[m], st_lo, st_hi, px.P, px.w, tr.vhat[m].w, &first,
                       &last);
    if (last < first) {
        first = 0x7fffffff;
        last = -1;
    }
}

// Warp-uniform parameters of the walk over one pair, kept in shared memory:
// the inner loop reads them only at anchors.
struct PairWalk {
    const double4_32a* txa;
    const double4_32a* txb;
    const float4* pq;
    int npa, npb, npp, n_pts;
};

// Shared memory of one block (one warp).
struct PairShared {
    PairChunk buf[2];
    PixelCtx px[kPThreads];
    PairWalk walk;
    unsigned long long stats[2];  // point evaluations, exact fallbacks
};

// One pixel tile (kPThreads pixels of the observer) against one slot of the
// trajectory set: the whole work of a block of the per-observer kernel, and
// one work item of the batched kernel.
template <bool PINGPONG, bool MULTI, bool REC>
__device__ __forceinline__ void pair_tile(const DevTraj& tr, const DevScreen& sc,
                                          const DevWork& wk, int slot, int tile,
                                          PairShared& sh) {
    const int pix = tile * kPThreads + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int np = sc.np;
    const bool active = pix < np;
    const int pc = active ? pix : np - 1;
    sh.px[threadIdx.x] = make_pixel(make_double3(sc.pix_pos[3 * pc], sc.pix_pos[3 * pc + 1],
                                                 sc.pix_pos[3 * pc + 2]),
                                    sc.pix_t0[pc], sc.dt, sc.nt);
    if (lane == 0) sh.stats[0] = sh.stats[1] = 0;
    const PixelCtx& px = sh.px[threadIdx.x];
    PairChunk* wb = sh.buf;
    PairWalk& W = sh.walk;
    PairSink sink;
    sink.init(static_cast<float*>(wk.scratch) + (int64_t)slot * wk.slot_stride +
              (int64_t)pc * sc.nt * 6);
    const int64_t g0 = wk.slot_seg[slot], g1 = wk.slot_seg[slot + 1];
    int j = g0 < g1 ? pair_of_segment(tr.pair_seg_offsets, tr.n_pairs, g0) : tr.n_pairs;
    // a slot holds at most 2048 particles of at most 2^31 points: the
    // per-thread deposit count stays below 2^32
    unsigned int inwin = 0;
    for (; j < tr.n_pairs && tr.pair_seg_offsets[j] < g1; ++j) {
        const int64_t sb = tr.pair_seg_offsets[j];
        const int64_t se = tr.pair_seg_offsets[j + 1];
        const int lg0 = (int)((g0 > sb ? g0 : sb) - sb);
        const int lg1 = (int)((g1 < se ? g1 : se) - sb);
        const int ma = 2 * j;
        const bool hasb = 2 * j + 1 < tr.n_particles;
        const int mb = hasb ? 2 * j + 1 : ma;
        const int npa = (int)(tr.offsets[ma + 1] - tr.offsets[ma]);
        const int npb = hasb ? (int)(tr.offsets[mb + 1] - tr.offsets[mb]) : 0;
        const int st_lo = lg0 << kSegShift;
        // the last point of a step of each particle in this slot (-1: none
        // for this lane)
        int lim_a = min(lg1 << kSegShift, npa - 1);
        int lim_b = hasb ? min(lg1 << kSegShift, npb - 1) : -1;
        int fa, la, fb, lb;
        particle_range(tr, ma, st_lo, lim_a, active, px, fa, la);
        particle_range(tr, mb, st_lo, hasb ? lim_b : st_lo, active, px, fb, lb);
        if (!active) lim_a = lim_b = -1;
        const int lo = warp_min(min(fa, fb)), hi = warp_max(max(la, lb));
        if (lo > hi) continue;  // uniform over the warp
        const int start = lo & ~(kPChunkLen - 1);  // >= st_lo, a segment boundary
        const int64_t po = tr.pair_offsets[j];
        const unsigned int lanes = __popc(__ballot_sync(0xffffffffu, active));
        if (lane == 0) {
            W.txa = tr.tx + tr.offsets[ma];
            W.txb = tr.tx + tr.offsets[mb];
            W.pq = tr.pq + kPairPoint * po;
            W.npa = npa;
            W.npb = npb;
            W.npp = (int)(tr.pair_offsets[j + 1] - po);
            W.n_pts = hi + 2 - start;  // points start .. hi+1
            sh.stats[0] += (unsigned long long)(hi + 2 - start) * (hasb ? 2u : 1u) * lanes;
        }
        __syncwarp();
        pair_stage(&wb[0], W.pq, start, min(kPChunkLen, W.npp - start), lane);
        Anchor2 A;
        PointState2 p1, p2;
        F2 comp = f2(0.0f, 0.0f), chain_err = f2(0.0f, 0.0f);  // chain_err includes A.err
        p2.rega = p2.regb = false;
        const int n_chunks = (W.n_pts + kPChunkLen - 1) >> kPChunkShift;
        for (int c = 0; c < n_chunks; c++) {
            const int p0 = start + (c << kPChunkShift);
            if (c + 1 < n_chunks) {
                pair_stage(&wb[(c + 1) & 1], W.pq, p0 + kPChunkLen,
                           min(kPChunkLen, W.npp - (p0 + kPChunkLen)), lane);
                asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            } else {
                asm volatile("cp.async.wait_group 0;\n" ::: "memory");
            }
            __syncwarp();
            const PairChunk& B = wb[c & 1];
            const bool anchor =
                c == 0 || (p0 & (kSegLen - 1)) == 0 ||
                warp_any_above(fmaxf(chain_err.v.x, chain_err.v.y), kReanchorBound);
            if (anchor) {
                Anchor aa, ab;
                // past its last point a particle repeats it, with positions
                // relative to that point's segment; a particle without points
                // borrows its partner's anchor (it never deposits)
                const int wa = W.npa, wbn = W.npb;
                const int ia = min(p0, wa - 1), ib = min(p0, wbn - 1);
                if (wa > 0) make_anchor(aa, W.txa[ia], W.txa[ia & ~(kSegLen - 1)], px, tr.frame);
                if (wbn > 0) make_anchor(ab, W.txb[ib], W.txb[ib & ~(kSegLen - 1)], px, tr.frame);
                else ab = aa;
                if (wa <= 0) aa = ab;
                const Anchor2 An = pack_anchor(aa, ab);
                if (c > 0) {
                    // rebase the chunk's previous point (in p2, see below):
                    // B + ki is unchanged
                    p2.ka += A.Ba - An.Ba;
                    p2.kb += A.Bb - An.Bb;
                }
                A = An;
            }
            const int n_here = min(kPChunkLen, W.n_pts - (c << kPChunkShift));
            // One step: point l of the chunk into q2, deposit q1 -> q2.  The
            // loop below alternates the roles of p1 and p2, so the point
            // state is never copied.
            auto step = [&](PointState2& q1, PointState2& q2, int l) {
                const int i = p0 + l;
                F2 aminus;
                point_field2(q2, B.p[l + 1], B.p[l], A, aminus);
                if (l == 0 && anchor) {
                    start_chain2(q2, A);
                    comp = f2(0.0f, 0.0f);
                    chain_err = A.err;
                } else {
                    const F2 du = step_increment2(q1, q2, aminus, B.p[l], f2(px.kdt, px.kdt));
                    chain_step2(q1, q2, du, comp);
                    chain_err = fma(f2(fabsf(du.v.x), fabsf(du.v.y)),
                                    f2(kChainRel, kChainRel), chain_err + f2(1.0e-7f, 1.0e-7f));
                }
                // the step ending at point i belongs to this lane and slot
                const bool dep_a = i > start && i <= lim_a;
                const bool dep_b = i > start && i <= lim_b;
                const int nt = sc.nt;
                const bool near_a = 0.5f - fabsf(q2.r.v.x) <= chain_err.v.x && i <= lim_a;
                const bool near_b = 0.5f - fabsf(q2.r.v.y) <= chain_err.v.y && i <= lim_b;
                q2.fla = 0;
                q2.flb = 0;
                q2.rega = !near_a && (unsigned)(A.Ba + q2.ka) < (unsigned)nt;
                q2.regb = !near_b && (unsigned)(A.Bb + q2.kb) < (unsigned)nt;
                if (near_a || near_b) {  // rare: one branch for both particles
                    if (near_a) {
                        const ExactPoint e = exact_point(W.txa, i, px, A.Ba);
                        q2.ka = e.ki;
                        q2.r.v.x = e.r;
                        q2.idxa = e.idx;
                        q2.fla = e.flags;
                        atomicAdd(&sh.stats[1], 1ull);
                    }
                    if (near_b) {
                        const ExactPoint e = exact_point(W.txb, i, px, A.Bb);
                        q2.kb = e.ki;
                        q2.r.v.y = e.r;
                        q2.idxb = e.idx;
                        q2.flb = e.flags;
                        atomicAdd(&sh.stats[1], 1ull);
                    }
                }
                if constexpr (REC) {
                    if (i <= lim_a) record_point<0>(wk, tr.n_particles, pix, ma, i, q2, A.Ba, nt);
                    if (i <= lim_b) record_point<1>(wk, tr.n_particles, pix, mb, i, q2, A.Bb, nt);
                }
                const bool fast_a = q1.rega && q2.rega && (unsigned)(q2.ka - q1.ka) <= 1u;
                const bool fast_b = q1.regb && q2.regb && (unsigned)(q2.kb - q1.kb) <= 1u;
                bool go_fast = __all_sync(0xffffffffu, (!dep_a || fast_a) && (!dep_b || fast_b));
                bool out_a = false, out_b = false;
                if (!go_fast) {
                    // steps that certainly lie outside the window add nothing
                    // and leave the fast path open
                    out_a = (q2.fla == 0 && A.Ba + q2.ka < 0) ||
                            (!(q1.fla & kExact) && A.Ba + q1.ka >= nt);
                    out_b = (q2.flb == 0 && A.Bb + q2.kb < 0) ||
                            (!(q1.flb & kExact) && A.Bb + q1.kb >= nt);
                    go_fast = __all_sync(0xffffffffu, (!dep_a || fast_a || out_a) &&
                                                          (!dep_b || fast_b || out_b));
                }
                // regular steps that span up to kMaxSpan bins beyond their first
                bool multi_a = false, multi_b = false, go_multi = false;
                if constexpr (MULTI) {
                    multi_a = q1.rega && q2.rega && (unsigned)(q2.ka - q1.ka) <= (unsigned)kMaxSpan;
                    multi_b = q1.regb && q2.regb && (unsigned)(q2.kb - q1.kb) <= (unsigned)kMaxSpan;
                    if (!go_fast)
                        go_multi = __all_sync(0xffffffffu, (!dep_a || multi_a || out_a) &&
                                                               (!dep_b || multi_b || out_b));
                }
                if (go_fast) {
                    const bool da = dep_a && fast_a, db = dep_b && fast_b;
                    // unconditional: a particle without a deposit adds zeros (its
                    // fields are finite for any observer off its trajectory)
                    deposit_fast2(q1, q2, A.Ba, A.Bb, da, db, sink);
                    inwin += (unsigned)da + (unsigned)db;
                } else if (go_multi) {
                    const bool da = dep_a && multi_a, db = dep_b && multi_b;
                    deposit_multi2(q1, q2, A.Ba, A.Bb, da, db, sink);
                    inwin += (unsigned)da + (unsigned)db;
                } else {
                    if (dep_a) {
                        PointState u1 = unpack<0>(q1), u2 = unpack<0>(q2);
                        materialize(u1, A.Ba, nt);
                        materialize(u2, A.Ba, nt);
                        PairView<0> v{&sink, nt};
                        if (deposit_step32(u1, u2, A.Ba, nt, v)) inwin++;
                    }
                    if (dep_b) {
                        PointState u1 = unpack<1>(q1), u2 = unpack<1>(q2);
                        materialize(u1, A.Bb, nt);
                        materialize(u2, A.Bb, nt);
                        PairView<1> v{&sink, nt};
                        if (deposit_step32(u1, u2, A.Bb, nt, v)) inwin++;
                    }
                }
            };
            if (PINGPONG) {
                // chunks are kPChunkLen (even) points long, so point l of every
                // chunk lives in p1 for even l and in p2 for odd l, and the
                // point before a chunk in p2
                for (int l = 0; l < n_here; l += 2) {
                    step(p2, p1, l);
                    if (l + 1 < n_here) step(p1, p2, l + 1);
                }
            } else {
                // one copy of the step body (fewer registers), the new point
                // copied into place after each step
                for (int l = 0; l < n_here; l++) {
                    step(p2, p1, l);
                    p2 = p1;
                }
            }
            __syncwarp();  // the buffer is restaged two chunks later
        }
    }
    sink.flush<0>();
    sink.flush<1>();
    if (sink.err) atomicOr(wk.status, sink.err);
    const unsigned long long win = warp_sum_u64(inwin);
    const unsigned long long nadd = warp_sum_u64(sink.n_add);
    __syncwarp();
    if (lane == 0 && wk.counters) {
        if (win) atomicAdd(wk.counters, win);
        if (sh.stats[1]) atomicAdd(wk.counters + 1, sh.stats[1]);
        if (nadd) atomicAdd(wk.counters + 2, nadd);
        if (sh.stats[0]) atomicAdd(wk.counters + 3, sh.stats[0]);
    }
}

// MAXREG: the register budget per thread, which sets how many one-warp
// blocks are resident per SM (65536 / (32 MAXREG)): 128 -> 16, 136 -> 15,
// 144 -> 14, 160 -> 13 (the unrolled loop needs ~152).  PINGPONG: the inner
// loop unrolled by two with alternating point states (no copies, more
// registers) or one step body with a copy per step.  MULTI: warps whose
// regular steps span up to kMaxSpan bins deposit them on packed pairs too
// (instead of per particle); for observers whose bins are short against the
// arrival advance of a step.  It costs ~1% where steps rarely span.
//
// REC: the recording instantiation, which also writes every point decision it
// takes into DevWork::rec (the parity tests compare them with the oracle's);
// its arithmetic and decisions are those of the instantiation without it.
template <int MAXREG, bool PINGPONG, bool MULTI = false, bool REC = false>
__global__ void __maxnreg__(MAXREG)
    lw_fp32_pair_kernel(DevTraj tr, DevScreen sc, DevWork wk) {
    __shared__ PairShared sh;
    pair_tile<PINGPONG, MULTI, REC>(tr, sc, wk, blockIdx.y, blockIdx.x, sh);
}

// Persistent form: every block takes (observer, tile, slot) items from the
// queue until it is empty.
template <int MAXREG, bool REC = false>
__global__ void __maxnreg__(MAXREG)
    lw_fp32_pair_batch_kernel(const DevTraj* trs, const DevScreen* scs, const DevWork* wks,
                              const BatchItem* items, int n_items, unsigned int* head) {
    __shared__ PairShared sh;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned int it = 0;
        if (lane == 0) it = atomicAdd(head, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= (unsigned int)n_items) break;
        const BatchItem bi = items[it];
        if (REC && wks[bi.obs].rec)
            pair_tile<false, false, true>(trs[bi.obs], scs[bi.obs], wks[bi.obs], bi.slot, bi.tile,
                                          sh);
        else
            pair_tile<false, false, false>(trs[bi.obs], scs[bi.obs], wks[bi.obs], bi.slot, bi.tile,
                                           sh);
        __syncwarp();
    }
}


cudaError_t launch_fp32_pair(const DevTraj& tr, const DevScreen& sc, const DevWork& w,
                             int variant, cudaStream_t s) {
    dim3 grid((sc.np + kPThreads - 1) / kPThreads, w.n_slots);
    if (w.rec) {
        // the recording instantiations of the kernels the automatic choice uses
        if (variant == kVariantPairMulti)
            lw_fp32_pair_kernel<128, false, true, true><<<grid, kPThreads, 0, s>>>(tr, sc, w);
        else if (variant == kVariantPair)
            lw_fp32_pair_kernel<128, false, false, true><<<grid, kPThreads, 0, s>>>(tr, sc, w);
        else
            return cudaErrorInvalidValue;
        return cudaGetLastError();
    }
    switch (variant) {
        case kVariantPair160:
            lw_fp32_pair_kernel<160, true><<<grid, kPThreads, 0, s>>>(tr, sc, w);
            break;
        case kVariantPair136:
            lw_fp32_pair_kernel<136, false><<<grid, kPThreads, 0, s>>>(tr, sc, w);
            break;
        case kVariantPair144:
            lw_fp32_pair_kernel<144, true><<<grid, kPThreads, 0, s>>>(tr, sc, w);
            break;
        case kVariantPairMulti:
            lw_fp32_pair_kernel<128, false, true><<<grid, kPThreads, 0, s>>>(tr, sc, w);
            break;
        default:
            lw_fp32_pair_kernel<128, false><<<grid, kPThreads, 0, s>>>(tr, sc, w);
            break;
    }
    return cudaGetLastError();
}

constexpr int kBatchMaxReg = 128;
int pair_batch_blocks_per_sm() { return 65536 / (32 * kBatchMaxReg); }

int pair_blocks_per_sm(int variant) {
    // occupancy of the kernel of each variant, asked once
    static int cached[5] = {-1, -1, -1, -1, -1};
    const int k = variant == kVariantPair160 ? 1 : variant == kVariantPair136 ? 2
                : variant == kVariantPair144 ? 3 : variant == kVariantPairMulti ? 4 : 0;
    if (cached[k] >= 0) return cached[k];
    int n = 0;
    cudaError_t e;
    switch (k) {
        case 1:
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lw_fp32_pair_kernel<160, true>,
                                                              kPThreads, 0);
            break;
        case 2:
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lw_fp32_pair_kernel<136, false>,
                                                              kPThreads, 0);
            break;
        case 3:
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lw_fp32_pair_kernel<144, true>,
                                                              kPThreads, 0);
            break;
        case 4:
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &n, lw_fp32_pair_kernel<128, false, true>, kPThreads, 0);
            break;
        default:
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, lw_fp32_pair_kernel<128, false>,
                                                              kPThreads, 0);
            break;
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cached[k] = n;
    return n;
}

cudaError_t launch_fp32_pair_batch(const DevTraj* trs, const DevScreen* scs, const DevWork* wks,
                                   const BatchItem* items, int n_items, unsigned int* head,
                                   int n_blocks, cudaStream_t s, bool record) {
    if (record)
        lw_fp32_pair_batch_kernel<kBatchMaxReg, true><<<n_blocks, kPThreads, 0, s>>>(
            trs, scs, wks, items, n_items, head);
    else
        lw_fp32_pair_batch_kernel<kBatchMaxReg><<<n_blocks, kPThreads, 0, s>>>(trs, scs, wks, items,
                                                                              n_items, head);
    return cudaGetLastError();
}

}  // namespace teufel
