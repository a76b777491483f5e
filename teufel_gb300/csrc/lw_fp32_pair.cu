// lw_fp32_pair.cu -- the split-precision kernel with two particles per
// thread.
//
// As the warp-uniform kernel (lw_fp32_warp.cu), each warp owns 32 pixels and
// walks trajectory points together, staged in shared memory.  Here every lane
// carries two particles (a pair of arrival neighbours) for its pixel, and all the
// per-point FP32 arithmetic -- the field, the arrival increment, the
// compensated chain and the deposit weights -- is done on packed pairs
// (add/sub/mul/fma.rn.f32x2), one instruction for both particles.  The
// trajectory data of a pair is interleaved component by component when the
// set is uploaded, so every operand pair comes straight out of shared memory.
// Bin decisions, fallbacks and the sink stay per particle.
//
// The step loop has one warp vote per step.  When every lane's steps are
// regular (both points resolved without the exact fallback, advancing by 0 or
// 1 bin, wherever they lie against the window), the warp deposits them on a
// straight-line path without branches; anything else -- a point within its
// error bound of a bin edge, or a step that spans several bins -- takes the
// general path, which is the reference's full case analysis
// (src/particle.cpp:786-865).
//
// The FP64-time instantiation (EXACT) takes the reference's FP64 arrival
// times, bins and bin edges for every point that can deposit, evaluated by
// the lanes of the warp in turn (ftime_resolve), with the FP32 chain deciding
// which points can.
//
// Each particle's open bin is implicit: the register accumulator of a
// particle always holds the not-yet-added contribution to the bin of its
// current point (B + k).  A step that leaves that bin adds the accumulator
// to the partial trace with fire-and-forget reductions and starts the next
// bin, so no bin index is carried or compared.  Both particles deposit into
// the lane's one pixel row.
#include <cuda_runtime.h>

#include <type_traits>

#include "lw_fp32_point.cuh"

namespace teufel {

// ---------------------------------------------------------------------------
// Preparation: the interleaved per-point data of every pair.
// ---------------------------------------------------------------------------
// A pair-point is kPairPoint float4, the two particles interleaved component
// by component (lo/hi halves: particle a, b):
//   0-1  e (offset from the segment's first point), dt of the step that ends here
//   2-3  beta^, 1 - |beta|
//   4-5  scaled beta', velocity-field scale
//   6-7  dA = beta^_i - c^_i, 1 - |beta_c| of the step that ends here
//   8-9  dB = beta^_i - c^_(i-1), unused
// all in the set's frame (c^_i: chord direction of the step i -> i+1).  dA and
// dB give the arrival-increment shares 1 - c^.N = (1 - beta^.N) + d.N of the
// point for the step that starts (dA) and the step that ends (dB) there, from
// the field's own 1 - beta^.N; they are formed in FP64, so their FP32 values
// carry full relative precision however small they are.  Everything the step
// ending at point i needs beyond the state of point i-1 lives in pair-point i.
__device__ __forceinline__ double3 unit_bg(const DevTraj& tr, int64_t q) {
    const double4_32a bg = tr.pp[q];
    const double P = sqrt(bg.x * bg.x + bg.y * bg.y + bg.z * bg.z);
    return P > 0.0 ? make_double3(bg.x / P, bg.y / P, bg.z / P) : make_double3(0.0, 0.0, 1.0);
}
// chord direction of the step q -> q+1 (the velocity direction where the step
// has no length)
__device__ __forceinline__ double3 chord_dir(const DevTraj& tr, int64_t q) {
    const double4_32a p = tr.tx[q], r = tr.tx[q + 1];
    const double ex = r.y - p.y, ey = r.z - p.z, ez = r.w - p.w;
    const double L = sqrt(ex * ex + ey * ey + ez * ez);
    return L > 0.0 ? make_double3(ex / L, ey / L, ez / L) : unit_bg(tr, q);
}

// The per-point data of point k (local index l) of a particle with points
// [o, o + n); beyond its last point (l >= n) the last point is repeated with
// a step of zero duration ending at it.
__device__ __forceinline__ void pair_point_data(const DevTraj& tr, int64_t o, int64_t n, int64_t l,
                                                float4& q0, float4& q1, float4& q2, float& dtp,
                                                float& cepsp, double3& dA, double3& dB) {
    const int64_t k = o + (l < n ? l : n - 1);
    q0 = tr.q0[k];
    q1 = tr.q1[k];
    q2 = tr.q2[k];
    const double3 b = unit_bg(tr, k);
    // the step starting here (none at the last point)
    const double3 cA = k + 1 < o + n ? chord_dir(tr, k) : b;
    dA = make_double3(b.x - cA.x, b.y - cA.y, b.z - cA.z);
    dtp = 0.0f;
    cepsp = 1.0f;
    dB = make_double3(0.0, 0.0, 0.0);
    if (l >= 1 && l < n) {
        // the step ending here: its duration, 1 - |chord velocity| and chord
        dtp = tr.q0[k - 1].w;
        cepsp = tr.q3[k - 1].w;
        const double3 cB = chord_dir(tr, k - 1);
        dB = make_double3(b.x - cB.x, b.y - cB.y, b.z - cB.z);
    }
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
    const int ma = tr.pair_members[2 * j];
    const int mb = tr.pair_members[2 * j + 1] >= 0 ? tr.pair_members[2 * j + 1] : ma;
    const int64_t oa = tr.offsets[ma], na = tr.offsets[ma + 1] - oa;
    const int64_t ob = tr.offsets[mb], nb = tr.offsets[mb + 1] - ob;
    float4 a0, a1, a2, b0, b1, b2;
    float dta = 0.0f, cea = 1.0f, dtb = 0.0f, ceb = 1.0f;
    double3 dAa = make_double3(0.0, 0.0, 0.0), dBa = dAa, dAb = dAa, dBb = dAa;
    if (na > 0) {
        pair_point_data(tr, oa, na, l, a0, a1, a2, dta, cea, dAa, dBa);
    } else {
        a0 = a1 = a2 = make_float4(0.0f, 0.0f, 1.0f, 1.0f);
    }
    if (nb > 0) {
        pair_point_data(tr, ob, nb, l, b0, b1, b2, dtb, ceb, dAb, dBb);
    } else {
        b0 = a0; b1 = a1; b2 = a2;
        dtb = dta; ceb = cea;
        dAb = dAa;
        dBb = dBa;
    }
    float4* o = pq + kPairPoint * i;
    o[0] = make_float4(a0.x, b0.x, a0.y, b0.y);
    o[1] = make_float4(a0.z, b0.z, dta, dtb);
    o[2] = make_float4(a1.x, b1.x, a1.y, b1.y);
    o[3] = make_float4(a1.z, b1.z, a1.w, b1.w);
    o[4] = make_float4(a2.x, b2.x, a2.y, b2.y);
    o[5] = make_float4(a2.z, b2.z, a2.w, b2.w);
    o[6] = make_float4((float)dAa.x, (float)dAb.x, (float)dAa.y, (float)dAb.y);
    o[7] = make_float4((float)dAa.z, (float)dAb.z, cea, ceb);
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
// The hardware approximations without the denormal handling of rsqrtf() and
// __fdividef(): no operand of these is ever subnormal (squared distances,
// 1 + beta^.N, kappa, sums of 1/R, step lengths in bins), and for normal
// operands the results are the same.
__device__ __forceinline__ float rsqrt_ftz(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rcp_ftz(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ F2 rsqrt2(F2 a) { return f2(rsqrt_ftz(a.v.x), rsqrt_ftz(a.v.y)); }
__device__ __forceinline__ F2 rcp2(F2 a) { return f2(rcp_ftz(a.v.x), rcp_ftz(a.v.y)); }
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

// The state of one point of a pair as the walk carries it.
struct PointState2 {
    int ka, kb;     // B + ka is the bin of particle a's point (likewise b)
    int exa, exb;   // 0, or rec_encode(bin, flags) of a point resolved exactly
    F2 r;           // the rest of (ts - t0)/dt - B - k, in [-1/2, 1/2] normally
    F2 iR;          // 1/|R|
    F2 aplus;       // 1 - c^.N with c^ the chord of the step this point starts
    F2 f[6];        // Ex, Ey, Ez, cBx, cBy, cBz
};
// with the FP64 arrival times of both points (the FP64-time mode)
struct PointState2T : PointState2 {
    double tsa, tsb;
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
// shares of the arrival increments: 1 - c^.N for the chord of the step that
// ends here (from dB, returned in aminus) and of the step that starts here
// (from dA, kept in S.aplus), as 1 - beta^.N + d.N.
__device__ __forceinline__ void point_field2(PointState2& S, const PairPoint& q, const Anchor2& A,
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
    aminus = a0 + dot(V2{lo2(q.d[8]), hi2(q.d[8]), lo2(q.d[9])}, N);
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
// state carries two numbers instead of N.  q is the pair-point the step ends
// at (its duration and chord 1 - |beta_c|).
__device__ __forceinline__ F2 step_increment2(const PointState2& p1, const PointState2& p2,
                                              F2 aminus, const PairPoint& q, F2 kdt) {
    const F2 ceps = hi2(q.d[7]);
    const F2 dt = hi2(q.d[1]);
    const F2 t = rcp2(p1.iR + p2.iR);
    const F2 one_m_cm = fma(p2.iR * t, p1.aplus, p1.iR * t * aminus);
    const F2 kap = fma(f2(1.0f, 1.0f) - ceps, one_m_cm, ceps);
    return dt * kdt * kap;
}

// Advance the compensated chain from p1 to p2 by du >= 0.  The integer part
// is split off by adding and subtracting 1.5 * 2^23, which rounds to the
// nearest integer (ties to even, as rintf) for |t| < 2^22; the integer is the
// low bits of t + 1.5 * 2^23.  Larger or non-finite t cannot pass the
// fallback test, whose bound grows with du: the point is then re-evaluated
// exactly.
constexpr float kRoundMagic = 12582912.0f;  // 1.5 * 2^23
__device__ __forceinline__ void chain_step2(const PointState2& p1, PointState2& p2, F2 du,
                                            F2& comp) {
    const F2 y = du - comp;
    const F2 t = p1.r + y;
    comp = (t - p1.r) - y;
    const F2 m = t + f2(kRoundMagic, kRoundMagic);
    const F2 k = m - f2(kRoundMagic, kRoundMagic);
    p2.r = t - k;
    p2.ka = p1.ka + (__float_as_int(m.v.x) - __float_as_int(kRoundMagic));
    p2.kb = p1.kb + (__float_as_int(m.v.y) - __float_as_int(kRoundMagic));
}

__device__ __forceinline__ void start_chain2(PointState2& S, const Anchor2& A) {
    const float kx = rintf(A.frac.v.x), ky = rintf(A.frac.v.y);
    S.ka = (int)kx;
    S.kb = (int)ky;
    S.r = A.frac - f2(kx, ky);
}

// One particle of a pair as a PointState for the general deposit, with its
// bin index and window flags: those of the exact evaluation where the point
// was resolved exactly, else those its bin implies.
template <int W>
__device__ __forceinline__ PointState unpack(const PointState2& S, int B, int nt) {
    PointState p;
    p.ki = W ? S.kb : S.ka;
    p.r = W ? S.r.v.y : S.r.v.x;
    const int ex = W ? S.exb : S.exa;
    if (ex) {
        p.idx = (ex & ((1 << kRecFlagShift) - 1)) - 4;
        p.flags = ex >> kRecFlagShift;
    } else {
        p.flags = 0;
        materialize(p, B, nt);
    }
#pragma unroll
    for (int c = 0; c < 3; c++)
        p.f[c] = W ? make_float2(S.f[2 * c].v.y, S.f[2 * c + 1].v.y)
                   : make_float2(S.f[2 * c].v.x, S.f[2 * c + 1].v.x);
    return p;
}

// The six components of one bin, added by three red.global.add.v2.f32 when p
// holds: the L2 adds them.  The reductions are issued under one branch rather
// than each under its own predicate, which the compiler would turn into three
// convergence regions.
__device__ __forceinline__ void red_add6_if(bool p, float* addr, float a0, float a1, float a2,
                                            float a3, float a4, float a5) {
    if (p)
        asm volatile(
            "red.global.add.v2.f32 [%0], {%1, %2};\n\t"
            "red.global.add.v2.f32 [%0+8], {%3, %4};\n\t"
            "red.global.add.v2.f32 [%0+16], {%5, %6};"
            ::"l"(addr), "f"(a0), "f"(a1), "f"(a2), "f"(a3), "f"(a4), "f"(a5)
            : "memory");
}

// The register accumulators of a lane: component c of particles a and b.
// acc holds, for each particle, what its current point's bin has received
// and not yet added to the partial trace (the pixel's row).
struct PairAcc {
    F2 acc[6];
    float* row;
    template <int W>
    __device__ __forceinline__ float get(int c) const {
        return W ? acc[c].v.y : acc[c].v.x;
    }
    template <int W>
    __device__ __forceinline__ void set(int c, float v) {
        if (W) acc[c].v.y = v; else acc[c].v.x = v;
    }
    template <int W>
    __device__ __forceinline__ void reduce_if(bool p, int k) {
        red_add6_if(p, row + (int64_t)k * 6, get<W>(0), get<W>(1), get<W>(2), get<W>(3),
                    get<W>(4), get<W>(5));
    }
    template <int W>
    __device__ __forceinline__ void clear() {
#pragma unroll
        for (int c = 0; c < 6; c++) set<W>(c, 0.0f);
    }
};

// The general deposit's sink for particle W: the reference's bin
// contributions in increasing bin order, merged in the accumulator while
// they go to one bin; `open` is the accumulator's bin (-1: none).
template <int W>
struct GeneralSink {
    PairAcc* a;
    int open;
    int nt;
    unsigned int* err;
    unsigned int* n_add;  // counts the contributions; nullptr: not counted here
    __device__ __forceinline__ void add(int k, const float2* f) {
        if (k < 0 || k >= nt) {
            *err |= 1u << TEUFEL_ERR_RANGE;
            return;
        }
        if (n_add) (*n_add)++;
        if (k == open) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                a->template set<W>(2 * c, a->template get<W>(2 * c) + f[c].x);
                a->template set<W>(2 * c + 1, a->template get<W>(2 * c + 1) + f[c].y);
            }
        } else {
            a->template reduce_if<W>(open >= 0, open);
            open = k;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                a->template set<W>(2 * c, f[c].x);
                a->template set<W>(2 * c + 1, f[c].y);
            }
        }
    }
};

// Regular steps of both particles (deposit_fast, lw_fp32_point.cuh, in packed
// form).  da/db: the particle deposits a regular step (k2 - k1 in {0, 1});
// ca/cb: its point leaves the bin of the step's start (for a particle that
// does not deposit, by any number of bins).  The step's trapezoid (fields f1,
// f2 at arrival r1 < r2 [bins]) is split at the bin edge when it crosses
// one: with dts = r2 - r1 (+1 on a crossing), a the part in bin k (dts when
// no crossing), lam = a/dts and fe = (1 - lam) f1 + lam f2,
//   bin k:   (f1 + fe) a/2       = f1 (2 - lam) a/2       + f2 lam a/2,
//   bin k+1: (fe + f2) (dts-a)/2 = f1 (1 - lam) (dts-a)/2 + f2 (1 + lam) (dts-a)/2.
// Bin k's part goes into the accumulator; on a crossing the accumulator is
// added to bin k (k1a/k1b: B + k of the step's start, v1a/v1b: inside the
// trace) and restarts with bin k+1's part.
__device__ __forceinline__ void deposit_fast2(const PointState2& p1, const PointState2& p2,
                                              bool da, bool db, bool ca, bool cb, int k1a,
                                              int k1b, bool v1a, bool v1b, PairAcc& s) {
    const F2 dts = f2(ca ? 1.0f : 0.0f, cb ? 1.0f : 0.0f) + (p2.r - p1.r);
    const F2 h = f2(0.5f, 0.5f) - p1.r;
    const F2 a = f2(ca ? h.v.x : dts.v.x, cb ? h.v.y : dts.v.y);
    const F2 q = a * rcp2(dts);
    // lam = 1 without a crossing or a deposit (dts may be zero there: a
    // particle past its last point repeats it)
    const F2 lam = f2(ca && da ? q.v.x : 1.0f, cb && db ? q.v.y : 1.0f);
    const F2 hw1 = f2(da ? 0.5f * a.v.x : 0.0f, db ? 0.5f * a.v.y : 0.0f);
    const F2 t2 = f2(0.5f, 0.5f) * (dts - a);  // zero without a crossing
    const F2 hw2 = f2(da ? t2.v.x : 0.0f, db ? t2.v.y : 0.0f);
    const F2 one = f2(1.0f, 1.0f);
    const F2 a1 = (f2(2.0f, 2.0f) - lam) * hw1, b1 = lam * hw1;
    const F2 a2 = (one - lam) * hw2, b2 = (one + lam) * hw2;
#pragma unroll
    for (int c = 0; c < 6; c++) s.acc[c] = fma(p2.f[c], b1, fma(p1.f[c], a1, s.acc[c]));
    // predicated reductions, no divergent branch
    s.reduce_if<0>(ca && v1a, k1a);
    s.reduce_if<1>(cb && v1b, k1b);
    const F2 keep = f2(ca ? 0.0f : 1.0f, cb ? 0.0f : 1.0f);
#pragma unroll
    for (int c = 0; c < 6; c++) s.acc[c] = fma(s.acc[c], keep, fma(p2.f[c], b2, p1.f[c] * a2));
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
    rd = rcp_ftz(dts);
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

// The multi-bin form of deposit_fast2: spa/spb >= 0 the bins a depositing
// particle's step spans beyond its first (0 for one that does not deposit).
// The first bin receives f1 a1 + f2 b1 and is added when the point leaves it;
// each full bin k1 + j, 0 < j < span, receives f1 w1(j) + f2 w2(j) with
// w1(j) = (u2 - j) rd, w2(j) = (j - u1) rd in bin units from k1 (u1 = r1,
// u2 = span + r2); the last bin starts with f1 a2 + f2 b2.
__device__ __forceinline__ void deposit_multi2(const PointState2& p1, const PointState2& p2,
                                               bool da, bool db, bool ca, bool cb, int k1a,
                                               int k1b, bool v1a, bool v1b, PairAcc& s) {
    const int spa = da ? p2.ka - p1.ka : 0, spb = db ? p2.kb - p1.kb : 0;
    float a1x, b1x, a2x, b2x, u2x, rdx, a1y, b1y, a2y, b2y, u2y, rdy;
    multi_weights(da, spa, p1.r.v.x, p2.r.v.x, a1x, b1x, a2x, b2x, u2x, rdx);
    multi_weights(db, spb, p1.r.v.y, p2.r.v.y, a1y, b1y, a2y, b2y, u2y, rdy);
    const F2 a1 = f2(a1x, a1y), b1 = f2(b1x, b1y), a2 = f2(a2x, a2y), b2 = f2(b2x, b2y);
    const F2 u1 = p1.r, u2 = f2(u2x, u2y), rd = f2(rdx, rdy);
#pragma unroll
    for (int c = 0; c < 6; c++) s.acc[c] = fma(p2.f[c], b1, fma(p1.f[c], a1, s.acc[c]));
    s.reduce_if<0>(ca && v1a, k1a);
    s.reduce_if<1>(cb && v1b, k1b);
    // full bins, in bin order per particle
    const int nfull = max(spa, spb) - 1;
    for (int j = 1; j <= nfull; j++) {
        const F2 jj = f2((float)j, (float)j);
        const F2 w1 = (u2 - jj) * rd, w2 = (jj - u1) * rd;
        F2 g[6];
#pragma unroll
        for (int c = 0; c < 6; c++) g[c] = fma(p2.f[c], w2, p1.f[c] * w1);
        const bool pa = j < spa, pb = j < spb;
        red_add6_if(pa, s.row + (int64_t)(k1a + j) * 6, g[0].v.x, g[1].v.x, g[2].v.x, g[3].v.x,
                    g[4].v.x, g[5].v.x);
        red_add6_if(pb, s.row + (int64_t)(k1b + j) * 6, g[0].v.y, g[1].v.y, g[2].v.y, g[3].v.y,
                    g[4].v.y, g[5].v.y);
    }
    const F2 keep = f2(ca ? 0.0f : 1.0f, cb ? 0.0f : 1.0f);
#pragma unroll
    for (int c = 0; c < 6; c++) s.acc[c] = fma(s.acc[c], keep, fma(p2.f[c], b2, p1.f[c] * a2));
}

// The reference's deposit of one step (src/particle.cpp:786-865) with the
// step's arrival times ts1, ts2 and the bin edges and centres in FP64, formed
// as the reference forms them (Geo64: t0 + (k +- 1/2) dt, t0 + k dt), and the
// fields in FP32.  Every difference of two of those times is exact in FP64
// (they lie within a few bins of each other); the weights -- such a
// difference over dts or dt -- are taken from it in FP32.  With the times
// bit-identical to the reference's, the deposit follows FP64's rounding of
// the arrival times, which on 1 as bins 30 m from the source is not
// negligible (a few 1e-6 bins per point).
template <class Sink>
__device__ __forceinline__ bool deposit_step_ftime(double ts1, double ts2, int idx1, int fl1,
                                                   int idx2, int fl2, const float2* f1,
                                                   const float2* f2, const Geo64& geo, float kdt,
                                                   int nt, Sink& sink) {
    if ((fl2 & kLeTmin) || !(fl1 & kLtTmax)) return false;
    const double dts = __dsub_rn(ts2, ts1);
    const float rdts = rcp_ftz((float)dts);
    if (idx2 > nt) idx2 = nt;
    float2 field[3];
    // f at time tq: weights w1 = (ts2 - tq)/dts, w2 = (tq - ts1)/dts
    auto interp = [&](double tq, float2* o) {
        const float2 w1 = splat2((float)__dsub_rn(ts2, tq) * rdts);
        const float2 w2 = splat2((float)__dsub_rn(tq, ts1) * rdts);
#pragma unroll
        for (int c = 0; c < 3; c++) o[c] = fma2(f1[c], w1, mul2(f2[c], w2));
    };
    // the last partial bin idx2: from its start to ts2
    auto last_bin = [&]() {
        const double tst = geo.start(idx2);
        interp(tst, field);
        const float2 wb = splat2(0.5f * (float)__dsub_rn(ts2, tst) * kdt);
#pragma unroll
        for (int c = 0; c < 3; c++) field[c] = mul2(add2(field[c], f2[c]), wb);
        sink.add(idx2, field);
    };
    if (fl1 & kLeTmin) {
        // the step starts before the window: bins 0 .. idx2-1 fully covered
        for (int k = 0; k < idx2; k++) {
            interp(geo.center(k), field);
            sink.add(k, field);
        }
        if (idx2 < nt) last_bin();
    } else if (idx1 == idx2) {
        // the step lies within one bin
        const float2 wb = splat2(0.5f * (float)dts * kdt);
#pragma unroll
        for (int c = 0; c < 3; c++) field[c] = mul2(add2(f1[c], f2[c]), wb);
        sink.add(idx1, field);
    } else {
        // first partial bin: from ts1 to its end
        const double te = geo.end(idx1);
        interp(te, field);
        const float2 wb = splat2(0.5f * (float)__dsub_rn(te, ts1) * kdt);
#pragma unroll
        for (int c = 0; c < 3; c++) field[c] = mul2(add2(f1[c], field[c]), wb);
        sink.add(idx1, field);
        for (int k = idx1 + 1; k < idx2; k++) {
            interp(geo.center(k), field);
            sink.add(k, field);
        }
        if (idx2 < nt) last_bin();
    }
    return true;
}

// The decision taken for point i of particle m (particle W of the pair) at
// this lane's pixel: the exact evaluation's bin and flags where the point
// fell back to it, else the bin B + k and the window flags it implies (as
// materialize does), into the decision record.  A point evaluated twice (the
// last point of one slot is the first of the next) must get the same
// decision both times; a difference is flagged.
template <int W>
__device__ __forceinline__ void record_point(const DevWork& wk, int n_particles, int pix, int m,
                                             int i, const PointState2& q, int B, int nt) {
    const int ex = W ? q.exb : q.exa;
    int v = ex;
    if (!ex) {
        int k = B + (W ? q.kb : q.ka);
        k = k < -2 ? -2 : (k > nt + 1 ? nt + 1 : k);
        v = rec_encode(k, (k < 0 ? kLeTmin : 0) | (k < nt ? kLtTmax : 0));
    }
    int* p = wk.rec + ((int64_t)pix * n_particles + m) * wk.rec_stride + i;
    const int old = atomicCAS(p, 0, v);
    if (old != 0 && old != v) atomicOr(p, kRecConflict);
}

// ---------------------------------------------------------------------------
// The kernel
// ---------------------------------------------------------------------------
constexpr int kPThreads = kPairTile;  // one warp per block: residency is set by registers alone

// Chunks of 16 pair-points: two staged chunks and the lanes' pixel data stay
// within 10 KB per block, so 16 one-warp blocks fit an SM's shared memory.
// Anchors may move at chunk boundaries; segment boundaries stay chunk
// boundaries.
// The chunk length is a template parameter CS (2^CS pair-points) the
// autotuner searches: 8, 16 (the default) or 32.
constexpr int kPChunkShift = 4;

// A staged chunk: p[l] is the chunk's point l.
template <int CS>
struct __align__(16) PairChunkT {
    static_assert(kSegLen % (1 << CS) == 0 && (1 << CS) % 2 == 0, "chunk layout");
    PairPoint p[1 << CS];
};

// The 32 lanes copy pair-points p0 .. p0+avail-1 of the pair whose data
// starts at pq.
template <int CS>
__device__ __forceinline__ void pair_stage(PairChunkT<CS>* b, const float4* pq, int p0, int avail,
                                           int lane) {
    const int n = kPairPoint * avail;
    const float4* src = pq + kPairPoint * (int64_t)p0;
    float4* dst = reinterpret_cast<float4*>(b->p);
#pragma unroll
    for (int k = 0; k < ((kPairPoint << CS) + 31) / 32; k++) {
        const int t = lane + 32 * k;
        if (t < n) {
            const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + t);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src + t)
                         : "memory");
        }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Staging by the bulk-copy (TMA) engine: lane 0 posts the expected byte
// count on the buffer's mbarrier and issues one cp.async.bulk of the whole
// chunk (its source in this GPU's memory, no multicast); every lane waits on
// the barrier's phase.  A chunk is avail * 160 bytes from a 16-byte aligned
// address, as the bulk copy requires.  Measured on the 1e5-particle screen
// (GB300, all parity tests passing on both): 675 ms per bench call against
// 636 ms with the lanes' 16-byte cp.async above, with or without the proxy
// fence, so the kernels stage with cp.async and this path is kept switched
// off for comparison.
constexpr bool kBulkStage = false;
__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_inval(unsigned long long* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
template <int CS>
__device__ __forceinline__ void bulk_stage(PairChunkT<CS>* b, const float4* pq, int p0, int avail,
                                           unsigned long long* bar) {
    const unsigned bytes = (unsigned)(avail * kPairPoint * sizeof(float4));
    unsigned long long src;
    asm("cvta.to.global.u64 %0, %1;" : "=l"(src) : "l"(pq + kPairPoint * (int64_t)p0));
    // the warp's earlier reads of this buffer (generic proxy) before the
    // copy's writes (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(b->p)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// Wait for phase `parity` of the barrier, for at most about a second of SM
// clock; false when it did not complete (the caller flags a timeout and
// stops waiting, so a lost copy cannot hang the kernel).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    const long long t_start = clock64();
    for (;;) {
        unsigned ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
        if (clock64() - t_start > (1ll << 31)) return false;
    }
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

// An FP64 arrival resolved for a lane: time and encoded decision.
struct FtimeResult {
    double ts;
    int ex;
    int pad;
};
// The FP64-time mode's per-step exchange: [kind][owner lane], kind 0/1 =
// points i-1 / i of particle a, 2/3 = of particle b.
struct FtimeShared {
    FtimeResult r[4][32];
};
struct NoFtimeShared {};

// Shared memory of one block (one warp).
template <int CS, bool EXACT = false>
struct PairSharedT {
    std::conditional_t<EXACT, FtimeShared, NoFtimeShared> ft;
    PairChunkT<CS> buf[2];
    PixelCtx px[kPThreads];
    int2 kstart[kPThreads];  // per lane: the bins (a, b) of the walk's first point
    PairWalk walk;
    unsigned long long stats[2];  // point evaluations, exact fallbacks
    unsigned long long bar[2];    // the buffers' bulk-copy barriers
};

// One pixel tile (kPThreads pixels of the observer) against one slot of the
// trajectory set: the whole work of a block of the per-observer kernel, and
// one work item of the batched kernel.
template <bool PINGPONG, bool MULTI, bool REC, bool EXACT = false, int CS = kPChunkShift>
__device__ __forceinline__ void pair_tile(const DevTraj& tr, const DevScreen& sc,
                                          const DevWork& wk, int slot, int tile,
                                          PairSharedT<CS, EXACT>& sh) {
    constexpr int kPChunkLen = 1 << CS;
    using PairChunk = PairChunkT<CS>;
    const int pix = tile * kPThreads + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int np = sc.np;
    const bool active = pix < np;
    const int pc = active ? pix : np - 1;
    sh.px[threadIdx.x] = make_pixel(make_double3(sc.pix_pos[3 * pc], sc.pix_pos[3 * pc + 1],
                                                 sc.pix_pos[3 * pc + 2]),
                                    sc.pix_t0[pc], sc.dt, sc.nt);
    if (lane == 0) sh.stats[0] = sh.stats[1] = 0;
    if (kBulkStage && lane == 0) {
        mbar_init(&sh.bar[0]);
        mbar_init(&sh.bar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // the phase each buffer's barrier completes next; set once a wait ran out
    unsigned phase = 0;
    bool stalled = false;
    __syncwarp();
    const PixelCtx& px = sh.px[threadIdx.x];
    const int nt = sc.nt;
    // bins this lane may add to: none for a lane without a pixel
    const unsigned nt_lane = active ? (unsigned)nt : 0u;
    PairChunk* wb = sh.buf;
    PairWalk& W = sh.walk;
    PairAcc s;
    s.row = static_cast<float*>(wk.scratch) + (int64_t)slot * wk.slot_stride +
            (int64_t)pc * nt * 6;
    unsigned int err = 0, n_add = 0;
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
        const int ma = tr.pair_members[2 * j];
        const bool hasb = tr.pair_members[2 * j + 1] >= 0;
        const int mb = hasb ? tr.pair_members[2 * j + 1] : ma;
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
        if constexpr (kBulkStage) {
            if (lane == 0 && !stalled)
                bulk_stage(&wb[0], W.pq, start, min(kPChunkLen, W.npp - start), &sh.bar[0]);
        } else {
            pair_stage(&wb[0], W.pq, start, min(kPChunkLen, W.npp - start), lane);
        }
        Anchor2 A{};  // made at the walk's first chunk
        using PS = std::conditional_t<EXACT, PointState2T, PointState2>;
        PS p1, p2;
        F2 comp = f2(0.0f, 0.0f), chain_err = f2(0.0f, 0.0f);  // chain_err includes A.err

        // The point is close enough to a bin edge that the estimate cannot
        // decide it (NaN-safe: a non-finite estimate falls back as well).
        auto near = [&](const PointState2& q) {
            const bool na = !(0.5f - fabsf(q.r.v.x) > chain_err.v.x);
            const bool nb = !(0.5f - fabsf(q.r.v.y) > chain_err.v.y);
            return make_int2(na, nb);
        };
        // the exact evaluation of point i of particle w
        auto resolve = [&](PointState2& q, int w, int i) {
            if (w == 0) {
                const ExactPoint e = exact_point(W.txa, i, px, A.Ba);
                q.ka = e.ki;
                q.r.v.x = e.r;
                q.exa = rec_encode(e.idx, e.flags);
            } else {
                const ExactPoint e = exact_point(W.txb, i, px, A.Bb);
                q.kb = e.ki;
                q.r.v.y = e.r;
                q.exb = rec_encode(e.idx, e.flags);
            }
            atomicAdd(&sh.stats[1], 1ull);
        };

        // Only steps that can reach the window resolve their points: the
        // FP32 chain places every point within chain_err (a few 1e-5) of its
        // bin coordinate, so a point whose chained bin is <= -2 lies before
        // tmin (bin edge -1/2), and one whose bin is >= nt + 1 at or after
        // tmax (edge nt - 1/2).  A step ending before the window or starting
        // after it deposits nothing (src/particle.cpp:793), and the
        // accumulator is then empty: arrivals increase along the walk.
        auto ftime_needed = [&](auto wtag, const auto& q1, const auto& q2, int i) {
            constexpr int Wp = decltype(wtag)::value;
            if (i > (Wp ? lim_b : lim_a)) return false;
            const int k1 = Wp ? A.Bb + q1.kb : A.Ba + q1.ka;
            const int k2 = Wp ? A.Bb + q2.kb : A.Ba + q2.ka;
            const bool sure = (Wp ? chain_err.v.y : chain_err.v.x) < 0.25f &&
                              fabsf(Wp ? q1.r.v.y : q1.r.v.x) <= 0.5f &&
                              fabsf(Wp ? q2.r.v.y : q2.r.v.x) <= 0.5f;
            return !(sure && (k2 <= -2 || k1 >= nt + 1));
        };
        // The FP64 evaluations the lanes need at this step (point i-1 of a
        // particle whose window opens here, point i of each particle whose
        // step can deposit), spread over the warp's lanes: an FP64
        // instruction costs the pipe as much for one active lane as for 32,
        // and most lanes need none at most steps.  Lane j evaluates the j-th
        // request (pixel from the shared pixel data, point from the
        // trajectory) and the owner takes the result from shared memory.
        auto ftime_resolve = [&](auto& q1, auto& q2, bool need_a, bool need_b, int i) {
            if constexpr (EXACT) {
                const bool lazy_a = need_a && !q1.exa, lazy_b = need_b && !q1.exb;
                unsigned m[4];
                m[0] = __ballot_sync(0xffffffffu, lazy_a);
                m[1] = __ballot_sync(0xffffffffu, need_a);
                m[2] = __ballot_sync(0xffffffffu, lazy_b);
                m[3] = __ballot_sync(0xffffffffu, need_b);
                const int c0 = __popc(m[0]), c1 = c0 + __popc(m[1]), c2 = c1 + __popc(m[2]);
                const int n = c2 + __popc(m[3]);
                for (int j = lane; j - lane < n; j += 32) {
                    if (j < n) {
                        const int kind = (j >= c0) + (j >= c1) + (j >= c2);
                        const int base = kind == 0 ? 0 : kind == 1 ? c0 : kind == 2 ? c1 : c2;
                        const int owner = (int)__fns(m[kind], 0, j - base + 1) & 31;
                        const PixelCtx& po = sh.px[owner];
                        const double ts = exact_retarded_time_fast(
                            (kind < 2 ? W.txa : W.txb)[i - 1 + (kind & 1)], po.P);
                        FtimeResult& res = sh.ft.r[kind][owner];
                        res.ts = ts;
                        res.ex = rec_encode(exact_bin_fast(ts, po.w, po.inv_dt),
                                            exact_flags(ts, po.w));
                    }
                }
                if (n == 0) return;
                __syncwarp();
                auto take = [&](auto& q, int w, int kind, int ip) {
                    const FtimeResult& res = sh.ft.r[kind][lane];
                    if (w) {
                        q.tsb = res.ts;
                        q.exb = res.ex;
                    } else {
                        q.tsa = res.ts;
                        q.exa = res.ex;
                    }
                    if constexpr (REC) {
                        if (w) record_point<1>(wk, tr.n_particles, pix, mb, ip, q, 0, nt);
                        else record_point<0>(wk, tr.n_particles, pix, ma, ip, q, 0, nt);
                    }
                };
                if (lazy_a) take(q1, 0, 0, i - 1);
                if (need_a) take(q2, 0, 1, i);
                if (lazy_b) take(q1, 1, 2, i - 1);
                if (need_b) take(q2, 1, 3, i);
                __syncwarp();  // the exchange is reused at the next step
            }
        };
        // The step q1 -> q2 of particle Wp with both points resolved.
        auto ftime_step = [&](auto wtag, auto& q1, auto& q2, int i) {
            constexpr int Wp = decltype(wtag)::value;
            const int e1 = Wp ? q1.exb : q1.exa, e2 = Wp ? q2.exb : q2.exa;
            const int idx1 = (e1 & ((1 << kRecFlagShift) - 1)) - 4;
            const int idx2 = (e2 & ((1 << kRecFlagShift) - 1)) - 4;
            const int fl1 = e1 >> kRecFlagShift;
            const int fl2 = e2 >> kRecFlagShift;
            float2 f1[3], f2[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                f1[c] = Wp ? make_float2(q1.f[2 * c].v.y, q1.f[2 * c + 1].v.y)
                           : make_float2(q1.f[2 * c].v.x, q1.f[2 * c + 1].v.x);
                f2[c] = Wp ? make_float2(q2.f[2 * c].v.y, q2.f[2 * c + 1].v.y)
                           : make_float2(q2.f[2 * c].v.x, q2.f[2 * c + 1].v.x);
            }
            // the accumulator belongs to the bin of q1 (when inside the trace)
            GeneralSink<Wp> g{&s, (unsigned)idx1 < nt_lane ? idx1 : -1, nt, &err, &n_add};
            const Geo64 geo{px.w.t0, px.w.dt};
            if (deposit_step_ftime(Wp ? q1.tsb : q1.tsa, Wp ? q2.tsb : q2.tsa, idx1, fl1, idx2,
                                   fl2, f1, f2, geo, px.kdt, nt, g))
                inwin++;
            const bool moved = g.open != idx2;
            s.reduce_if<Wp>(moved && g.open >= 0, g.open);
            if (moved) s.clear<Wp>();
        };
        const std::integral_constant<int, 0> kPa;
        const std::integral_constant<int, 1> kPb;

        // One step: point l of the chunk into q2 (the chain continued from q1,
        // or started afresh at a new anchor), then the step q1 -> q2 deposited.
        auto step = [&](auto fresh, PS& q1, PS& q2, const PairChunk& B, int l, int i) {
            F2 aminus;
            point_field2(q2, B.p[l], A, aminus);
            q2.exa = q2.exb = 0;
            if constexpr (decltype(fresh)::value) {
                start_chain2(q2, A);
                comp = f2(0.0f, 0.0f);
                chain_err = A.err;
            } else {
                const F2 du = step_increment2(q1, q2, aminus, B.p[l], f2(px.kdt, px.kdt));
                chain_step2(q1, q2, du, comp);
                // du >= 0: arrivals increase along the points
                chain_err = fma(du, f2(kChainRel, kChainRel), chain_err + f2(1.0e-7f, 1.0e-7f));
            }
            if constexpr (EXACT) {
                // FP32 fields, the reference's FP64 arrival times: the bin and
                // flags of every point that can deposit are the reference's
                const bool need_a = ftime_needed(kPa, q1, q2, i);
                const bool need_b = ftime_needed(kPb, q1, q2, i);
                ftime_resolve(q1, q2, need_a, need_b, i);
                if (need_a) ftime_step(kPa, q1, q2, i);
                if (need_b) ftime_step(kPb, q1, q2, i);
                return;
            }
            // the step ending at point i belongs to this lane and slot
            const bool dep_a = i <= lim_a, dep_b = i <= lim_b;
            const int2 nr = near(q2);
            const int k1a = A.Ba + q1.ka, k1b = A.Bb + q1.kb;
            const int k2a = A.Ba + q2.ka, k2b = A.Bb + q2.kb;
            // Regular: resolved without the fallback, advancing by at most one
            // bin.  Wherever such a step lies, the fast deposit is the
            // reference's: inside the window; entering it (bin -1 to 0) it puts
            // into bin 0 the part after the edge, as the reference's branch for
            // a step that starts before the window does; leaving it (bin nt-1
            // to nt) it puts into bin nt-1 the part before the edge (the
            // reference caps the last bin at nt and adds nothing there); and
            // what falls in bins outside [0, nt) stays in the accumulator, which
            // is never added to the trace for such a bin.
            const bool fast_a = q1.exa == 0 && !nr.x && (unsigned)(q2.ka - q1.ka) <= 1u;
            const bool fast_b = q1.exb == 0 && !nr.y && (unsigned)(q2.kb - q1.kb) <= 1u;
            const bool ok_a = !dep_a || fast_a;
            const bool ok_b = !dep_b || fast_b;
            const bool ca = q2.ka != q1.ka, cb = q2.kb != q1.kb;
            const bool v1a = (unsigned)k1a < nt_lane, v1b = (unsigned)k1b < nt_lane;
            bool go_multi = false;
            bool multi_a = false, multi_b = false;
            const bool go_fast = __all_sync(0xffffffffu, ok_a && ok_b);
            if constexpr (MULTI) {
                // bins inside the trace, or certainly outside the window
                const bool r1a = q1.exa == 0 && (unsigned)k1a < (unsigned)nt;
                const bool r1b = q1.exb == 0 && (unsigned)k1b < (unsigned)nt;
                const bool r2a = !nr.x && (unsigned)k2a < (unsigned)nt;
                const bool r2b = !nr.y && (unsigned)k2b < (unsigned)nt;
                const bool out_a = (!nr.x && k2a < 0) || (q1.exa == 0 && k1a >= nt);
                const bool out_b = (!nr.y && k2b < 0) || (q1.exb == 0 && k1b >= nt);
                multi_a = r1a && r2a && (unsigned)(q2.ka - q1.ka) <= (unsigned)kMaxSpan;
                multi_b = r1b && r2b && (unsigned)(q2.kb - q1.kb) <= (unsigned)kMaxSpan;
                if (!go_fast)
                    go_multi = __all_sync(0xffffffffu,
                                          (!dep_a || (!nr.x && (multi_a || out_a))) &&
                                              (!dep_b || (!nr.y && (multi_b || out_b))));
            }
            if (go_fast) {
                const bool da = dep_a && fast_a, db = dep_b && fast_b;
                deposit_fast2(q1, q2, da, db, ca, cb, k1a, k1b, v1a, v1b, s);
                // the steps the reference deposits (ts2 > tmin, ts1 < tmax); the
                // bins they add to are counted once per walk
                const bool ia = da && k2a >= 0 && k1a < nt, ib = db && k2b >= 0 && k1b < nt;
                inwin += (unsigned)ia + (unsigned)ib;
            } else if (go_multi) {
                const bool da = dep_a && multi_a, db = dep_b && multi_b;
                deposit_multi2(q1, q2, da, db, ca, cb, k1a, k1b, v1a, v1b, s);
                inwin += (unsigned)da + (unsigned)db;
            } else {
                // the general path: exact fallbacks, then the reference's
                // deposit per particle through the accumulator of its bin
                if (dep_a && nr.x) resolve(q2, 0, i);
                if (dep_b && nr.y) resolve(q2, 1, i);
                {
                    GeneralSink<0> g{&s, v1a ? k1a : -1, nt, &err, nullptr};
                    if (dep_a) {
                        const PointState u1 = unpack<0>(q1, A.Ba, nt), u2 = unpack<0>(q2, A.Ba, nt);
                        if (deposit_step32(u1, u2, A.Ba, nt, g)) inwin++;
                    }
                    // the accumulator belongs to the bin of the new point
                    const bool moved = g.open != A.Ba + q2.ka;
                    s.reduce_if<0>(moved && g.open >= 0, g.open);
                    if (moved) s.clear<0>();
                }
                {
                    GeneralSink<1> g{&s, v1b ? k1b : -1, nt, &err, nullptr};
                    if (dep_b) {
                        const PointState u1 = unpack<1>(q1, A.Bb, nt), u2 = unpack<1>(q2, A.Bb, nt);
                        if (deposit_step32(u1, u2, A.Bb, nt, g)) inwin++;
                    }
                    const bool moved = g.open != A.Bb + q2.kb;
                    s.reduce_if<1>(moved && g.open >= 0, g.open);
                    if (moved) s.clear<1>();
                }
            }
            if constexpr (REC) {
                if (dep_a) record_point<0>(wk, tr.n_particles, pix, ma, i, q2, A.Ba, nt);
                if (dep_b) record_point<1>(wk, tr.n_particles, pix, mb, i, q2, A.Bb, nt);
            }
        };

        const std::integral_constant<bool, true> kFresh;
        const std::integral_constant<bool, false> kChained;
        const int n_chunks = (W.n_pts + kPChunkLen - 1) >> CS;
        for (int c = 0; c < n_chunks; c++) {
            const int p0 = start + (c << CS);
            if constexpr (kBulkStage) {
                if (c + 1 < n_chunks && lane == 0 && !stalled)
                    bulk_stage(&wb[(c + 1) & 1], W.pq, p0 + kPChunkLen,
                               min(kPChunkLen, W.npp - (p0 + kPChunkLen)), &sh.bar[(c + 1) & 1]);
                const int b = c & 1;
                if (!stalled && !mbar_wait(&sh.bar[b], (phase >> b) & 1u)) {
                    stalled = true;
                    err |= 1u << TEUFEL_ERR_TIMEOUT;
                }
                phase ^= 1u << b;
                stalled = __any_sync(0xffffffffu, stalled);
            } else {
                if (c + 1 < n_chunks) {
                    pair_stage(&wb[(c + 1) & 1], W.pq, p0 + kPChunkLen,
                               min(kPChunkLen, W.npp - (p0 + kPChunkLen)), lane);
                    asm volatile("cp.async.wait_group 1;\n" ::: "memory");
                } else {
                    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
                }
            }
            __syncwarp();
            const PairChunk& B = wb[c & 1];
            // (the FP64-time mode needs the chain only to a fraction of a bin)
            const bool anchor =
                c == 0 || (p0 & (kSegLen - 1)) == 0 ||
                warp_any_above(fmaxf(chain_err.v.x, chain_err.v.y),
                               EXACT ? 0.01f : kReanchorBound);
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
                    // rebase the previous point: B + k is unchanged
                    p1.ka += A.Ba - An.Ba;
                    p1.kb += A.Bb - An.Bb;
                }
                A = An;
            }
            const int n_here = min(kPChunkLen, W.n_pts - (c << CS));
            int l = 0;
            if (c == 0) {
                // the walk's first point: no step ends there
                F2 aminus;
                point_field2(p1, B.p[0], A, aminus);
                p1.exa = p1.exb = 0;
                start_chain2(p1, A);
                comp = f2(0.0f, 0.0f);
                chain_err = A.err;
                if constexpr (EXACT) {
                    // resolved by the first step that can deposit
                } else {
                    const int2 nr = near(p1);
                    if (nr.x && start <= lim_a) resolve(p1, 0, start);
                    if (nr.y && start <= lim_b) resolve(p1, 1, start);
                    sh.kstart[threadIdx.x] = make_int2(A.Ba + p1.ka, A.Bb + p1.kb);
                }
                if constexpr (REC && !EXACT) {
                    if (start <= lim_a)
                        record_point<0>(wk, tr.n_particles, pix, ma, start, p1, A.Ba, nt);
                    if (start <= lim_b)
                        record_point<1>(wk, tr.n_particles, pix, mb, start, p1, A.Bb, nt);
                }
#pragma unroll
                for (int q = 0; q < 6; q++) s.acc[q] = f2(0.0f, 0.0f);
                l = 1;
            } else if (anchor) {
                step(kFresh, p1, p2, B, 0, p0);
                p1 = p2;
                l = 1;
            }
            if (PINGPONG) {
                // two steps per trip with the roles of the point states
                // alternating: no copy of the state
                for (; l + 1 < n_here; l += 2) {
                    step(kChained, p1, p2, B, l, p0 + l);
                    step(kChained, p2, p1, B, l + 1, p0 + l + 1);
                }
                if (l < n_here) {
                    step(kChained, p1, p2, B, l, p0 + l);
                    p1 = p2;
                }
            } else {
                // one copy of the step body (fewer registers), the new point
                // copied into place after each step
                for (; l < n_here; l++) {
                    step(kChained, p1, p2, B, l, p0 + l);
                    p1 = p2;
                }
            }
            __syncwarp();  // the buffer is restaged two chunks later
        }
        // what the accumulators still hold belongs to the bins of the walk's
        // last point
        {
            // (FP64-time mode: the bins of the resolved point; an unresolved
            // one ends a walk whose accumulator is empty)
            const int ka = EXACT ? (p1.exa ? (p1.exa & ((1 << kRecFlagShift) - 1)) - 4 : -1)
                                 : A.Ba + p1.ka;
            const int kb = EXACT ? (p1.exb ? (p1.exb & ((1 << kRecFlagShift) - 1)) - 4 : -1)
                                 : A.Bb + p1.kb;
            s.reduce_if<0>((unsigned)ka < nt_lane, ka);
            s.reduce_if<1>((unsigned)kb < nt_lane, kb);
            if constexpr (!EXACT) {
                // Bins the walk added to beyond one per in-window step: its
                // arrivals increase, and every step adds to each bin of the
                // trace between its end points' bins (the reference's
                // partial, full and partial bins), so over the walk they are
                // the bin edges inside the trace crossed between its first
                // and its last point.  Every point the walk reaches is one of
                // the particle's steps in this slot, or its repeated last point.
                const int2 k0 = sh.kstart[threadIdx.x];
                if (lim_a >= 0) n_add += (unsigned)max(0, min(ka, nt - 1) - max(k0.x, 0));
                if (lim_b >= 0) n_add += (unsigned)max(0, min(kb, nt - 1) - max(k0.y, 0));
            }
        }
    }
    if (kBulkStage) {
        // every copy issued was waited for (unless a wait ran out)
        __syncwarp();
        if (lane == 0) {
            mbar_inval(&sh.bar[0]);
            mbar_inval(&sh.bar[1]);
        }
    }
    if (err) atomicOr(wk.status, err);
    const unsigned long long win = warp_sum_u64(inwin);
    // deposits: per in-window step one bin, plus the edges crossed
    const unsigned long long nadd = warp_sum_u64(EXACT ? n_add : n_add + inwin);
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
// 144 -> 14, 160 -> 13.  PINGPONG: the inner loop unrolled by two with
// alternating point states (no copies, more registers) or one step body with
// a copy per step.  MULTI: warps whose regular steps span up to kMaxSpan bins
// deposit them on packed pairs too (instead of per particle); for observers
// whose bins are short against the arrival advance of a step.
//
// REC: the recording instantiation, which also writes every point decision it
// takes into DevWork::rec (the parity tests compare them with the oracle's);
// its arithmetic and decisions are those of the instantiation without it.
//
// EXACT: the FP64-time mode (FP32 fields, the reference's FP64 arrival times,
// bins and bin edges), for observers whose bins are so short that FP64's own
// rounding of the arrival times is not negligible against them.
//
// CS: chunks of 2^CS pair-points (8, 16 or 32).
template <int MAXREG, bool PINGPONG, bool MULTI = false, bool REC = false, bool EXACT = false,
          int CS = kPChunkShift>
__global__ void __maxnreg__(MAXREG)
    lw_fp32_pair_kernel(DevTraj tr, DevScreen sc, DevWork wk) {
    __shared__ PairSharedT<CS, EXACT> sh;
    pair_tile<PINGPONG, MULTI, REC, EXACT, CS>(tr, sc, wk, blockIdx.y, blockIdx.x, sh);
}

// Persistent form: every block takes (observer, tile, slot) items from the
// queue until it is empty.
template <int MAXREG, bool REC = false>
__global__ void __maxnreg__(MAXREG)
    lw_fp32_pair_batch_kernel(const DevTraj* trs, const DevScreen* scs, const DevWork* wks,
                              const BatchItem* items, int n_items, unsigned int* head) {
    __shared__ PairSharedT<kPChunkShift> sh;
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
        else if (variant == kVariantPairTime)
            lw_fp32_pair_kernel<128, false, false, true, true><<<grid, kPThreads, 0, s>>>(tr, sc,
                                                                                        w);
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
        case kVariantPairTime:
            lw_fp32_pair_kernel<128, false, false, false, true><<<grid, kPThreads, 0, s>>>(tr, sc,
                                                                                         w);
            break;
        case kVariantPairC8:
            lw_fp32_pair_kernel<128, false, false, false, false, 3><<<grid, kPThreads, 0, s>>>(
                tr, sc, w);
            break;
        case kVariantPairC32:
            lw_fp32_pair_kernel<128, false, false, false, false, 5><<<grid, kPThreads, 0, s>>>(
                tr, sc, w);
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
    static int cached[8] = {-1, -1, -1, -1, -1, -1, -1, -1};
    const int k = variant == kVariantPair160 ? 1 : variant == kVariantPair136 ? 2
                : variant == kVariantPair144 ? 3 : variant == kVariantPairMulti ? 4
                : variant == kVariantPairTime ? 5 : variant == kVariantPairC8 ? 6
                : variant == kVariantPairC32 ? 7 : 0;
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
        case 5:
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &n, lw_fp32_pair_kernel<128, false, false, false, true>, kPThreads, 0);
            break;
        case 6:
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &n, lw_fp32_pair_kernel<128, false, false, false, false, 3>, kPThreads, 0);
            break;
        case 7:
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                &n, lw_fp32_pair_kernel<128, false, false, false, false, 5>, kPThreads, 0);
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
