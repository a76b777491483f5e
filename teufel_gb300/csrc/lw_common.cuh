// lw_common.cuh -- device functions shared by the FP64 and the FP32-split
// field-integration kernels.
//
// Everything that decides WHERE a trajectory step lands in a trace -- the
// retarded time, the bin index round((ts - t0)/dt), and the window tests
// against tmin/tmax -- is evaluated here with IEEE-rounded double intrinsics
// (__dadd_rn, __dmul_rn, __ddiv_rn, __dsqrt_rn), which the compiler never
// contracts into FMAs.  Given the same inputs this reproduces the reference's
// values bit for bit:
//   RetardedTime      src/particle.cpp:560-568   (t + |obs - x| / c)
//   Vector::norm      src/vector.cpp:136-139     (sqrt(x*x + y*y + z*z))
//   window, indices   src/particle.cpp:780-781, 805, 831, 833
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "lw_internal.h"
#include "teufel_cuda.h"

namespace teufel {

// point flags
constexpr int kLeTmin = 1;   // ts <= tmin  (the step starting here begins before the window)
constexpr int kLtTmax = 2;   // ts <  tmax
constexpr int kExact = 4;    // resolved by the exact FP64 evaluation

struct Window {
    double t0, dt, tmin, tmax;
    int nt;
};

__device__ __forceinline__ Window make_window(double t0, double dt, int nt) {
    Window w;
    w.t0 = t0;
    w.dt = dt;
    w.nt = nt;
    // tmin = t0 - dt*0.5; tmax = t0 + dt*((double)nots - 0.5)  (src/particle.cpp:780-781)
    w.tmin = __dsub_rn(t0, __dmul_rn(dt, 0.5));
    w.tmax = __dadd_rn(t0, __dmul_rn(dt, __dsub_rn((double)nt, 0.5)));
    return w;
}

// The reference's retarded time of one trajectory point, bit-exact.
__device__ __forceinline__ double exact_retarded_time(const double4_32a tx, const double3 obs) {
    double rx = __dsub_rn(obs.x, tx.y);
    double ry = __dsub_rn(obs.y, tx.z);
    double rz = __dsub_rn(obs.z, tx.w);
    double r2 = __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz));
    double R = __dsqrt_rn(r2);
    return __dadd_rn(tx.x, __ddiv_rn(R, kC));
}

// a / b rounded to nearest for a divisor with a known reciprocal y = RN(1/b),
// in fewer FP64 operations than the IEEE division: q0 = RN(a y) lies within
// two ulps of a/b, the residual a - q0 b is formed by an FMA, and one
// correction step q1 = RN(q0 + r y) (Markstein's, 1990) gives the rounded
// quotient in all but rare cases.  q1 is returned only when its own residual
// proves it: a - q1 b is exact in an FMA for a q1 next to a/b, and
// |a - q1 b| < |b| ulp(q1)/2 (1 - 2^-20) puts a/b strictly within half a
// spacing of q1 on both sides (q1 not a power of two, whose lower spacing is
// half as wide).  Otherwise -- near a rounding tie, subnormal, huge or
// non-finite values -- the IEEE division decides.
__device__ __forceinline__ double div_rn_by(double a, double b, double y) {
    const double q0 = __dmul_rn(a, y);
    const double q1 = __fma_rn(__fma_rn(-q0, b, a), y, q0);
    const double r1 = __fma_rn(-q1, b, a);
    const unsigned long long bits = (unsigned long long)__double_as_longlong(q1);
    const unsigned long long ex = bits & 0x7ff0000000000000ULL;
    // ulp(q1) = 2^(e - 52) for exponent fields e in (53, 2047)
    if (ex > (53ULL << 52) && ex < 0x7ff0000000000000ULL && (bits & 0x000fffffffffffffULL)) {
        const double ulp = __longlong_as_double((long long)(ex - (52ULL << 52)));
        if (fabs(r1) < fabs(b) * ulp * (0.5 * (1.0 - 0x1p-20))) return q1;
    }
    return __ddiv_rn(a, b);
}

// exact_retarded_time with R/c through div_rn_by: the same double.
__device__ __forceinline__ double exact_retarded_time_fast(const double4_32a tx,
                                                           const double3 obs) {
    double rx = __dsub_rn(obs.x, tx.y);
    double ry = __dsub_rn(obs.y, tx.z);
    double rz = __dsub_rn(obs.z, tx.w);
    double r2 = __dadd_rn(__dadd_rn(__dmul_rn(rx, rx), __dmul_rn(ry, ry)), __dmul_rn(rz, rz));
    double R = __dsqrt_rn(r2);
    return __dadd_rn(tx.x, div_rn_by(R, kC, 1.0 / kC));
}

// Bin index of an exact arrival time, clamped to [-2, nt+1].  The clamp keeps
// every decision the deposit takes (indices below 0 only matter through the
// tmin flag, indices above nt are capped to nt by the reference, :806, :834).
__device__ __forceinline__ int exact_bin(double ts, const Window& w) {
    double u = __ddiv_rn(__dsub_rn(ts, w.t0), w.dt);
    u = fmax(-4.0, fmin(u, (double)w.nt + 4.0));
    int k = (int)round(u);  // round(): half away from zero, as C's round()
    return k < -2 ? -2 : (k > w.nt + 1 ? w.nt + 1 : k);
}

// exact_bin with the quotient replaced by a product with inv_dt = RN(1/dt):
// the two differ by at most two ulps, so they round to the same integer
// unless the product lies within 1e-9 of a half-integer (then the IEEE
// quotient decides).  The same bin for |(ts - t0)/dt| < 2^20.
__device__ __forceinline__ int exact_bin_fast(double ts, const Window& w, double inv_dt) {
    const double d = __dsub_rn(ts, w.t0);
    double u = __dmul_rn(d, inv_dt);
    const double k = round(u);
    if (!(fabs(u - k) < 0.5 - 1e-9) || !(fabs(u) < 1048576.0)) u = __ddiv_rn(d, w.dt);
    u = fmax(-4.0, fmin(u, (double)w.nt + 4.0));
    const int ki = (int)round(u);
    return ki < -2 ? -2 : (ki > w.nt + 1 ? w.nt + 1 : ki);
}

__device__ __forceinline__ int exact_flags(double ts, const Window& w) {
    return (ts <= w.tmin ? kLeTmin : 0) | (ts < w.tmax ? kLtTmax : 0) | kExact;
}

// Fast arrival-time estimate for range searches only (FMA, approximate sqrt):
// within a few ulp of the larger of its terms t and R/c; callers widen
// ranges by two steps.  mag (optional) receives |t| + R/c, the scale of its
// rounding: when t is close to -R/c (a negative emission time) the sum is
// much smaller than its terms and carries their rounding, not its own.
__device__ __forceinline__ double approx_retarded_time(const double4_32a tx, const double3 obs,
                                                       double* mag = nullptr) {
    double rx = obs.x - tx.y, ry = obs.y - tx.z, rz = obs.z - tx.w;
    double r2 = fma(rx, rx, fma(ry, ry, rz * rz));
    const double rc = sqrt(r2) * (1.0 / kC);
    if (mag) *mag = fabs(tx.x) + rc;
    return fma(sqrt(r2), 1.0 / kC, tx.x);
}

// In-window step range of one particle for one observer, found by bisection
// on the (monotone) arrival time over steps [st_lo, st_hi).  Returns the
// first and last step that may overlap [tmin, tmax]; an empty range has
// first > last.  Widened by two steps on each side against rounding; the
// per-step exact decisions then select exactly the reference's steps.
// min_inc: the particle's smallest arrival advance of a step (vhat.w).  The
// bisection needs the computed arrival times to increase along the points;
// they do when that advance exceeds their rounding, checked here against 64
// ulps of the scale of their terms, |t| + R/c, at the ends of the range
// (emission times and distances between those ends are bounded by theirs for
// a forward, slower-than-light trajectory: |t| by the larger end, R/c by the
// larger end plus the time between the ends).  Otherwise the whole range is
// returned.
__device__ __forceinline__ void inwindow_steps(const double4_32a* tx, int st_lo, int st_hi,
                                               const double3 obs, const Window& w,
                                               double min_inc, int* first, int* last) {
    double mag_lo, mag_hi;
    const double ts_lo = approx_retarded_time(tx[st_lo], obs, &mag_lo);
    const double ts_hi = approx_retarded_time(tx[st_hi], obs, &mag_hi);
    const double span = fabs(tx[st_hi].x - tx[st_lo].x);
    if (!(min_inc > 64.0 * 2.220446049250313e-16 * (fmax(mag_lo, mag_hi) + span))) {
        *first = st_lo;
        *last = st_hi - 1;
        return;
    }
    // first point with ts > tmin in [st_lo, st_hi]; one evaluation when the
    // window opens before the range does
    int lo = st_lo, hi = st_hi + 1;
    if (ts_lo > w.tmin) hi = lo;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (approx_retarded_time(tx[mid], obs) > w.tmin) hi = mid; else lo = mid + 1;
    }
    int i_first = lo;
    // last point with ts < tmax in [st_lo, st_hi]; one evaluation when the
    // window closes after the range does
    lo = st_lo - 1;
    hi = st_hi;
    if (ts_hi < w.tmax) lo = hi;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (approx_retarded_time(tx[mid], obs) < w.tmax) lo = mid; else hi = mid - 1;
    }
    int j_last = lo;
    int f = i_first - 1 - 2;
    int l = j_last + 2;
    *first = f < st_lo ? st_lo : f;
    *last = l > st_hi - 1 ? st_hi - 1 : l;
}

// ---------------------------------------------------------------------------
// Arithmetic policy of the generic deposit: IEEE-rounded FP64 operations in
// the reference's order (the FP32 path has its own deposit_step32).
// ---------------------------------------------------------------------------
struct Ops64 {
    typedef double T;
    __device__ static T add(T a, T b) { return __dadd_rn(a, b); }
    __device__ static T sub(T a, T b) { return __dsub_rn(a, b); }
    __device__ static T mul(T a, T b) { return __dmul_rn(a, b); }
    __device__ static T div(T a, T b) { return __ddiv_rn(a, b); }
};
// Time coordinates of the bins.  Geo64 works in seconds exactly as the
// reference (t_center = t0 + idx*dt etc., src/particle.cpp:812, 816, 845,
// 851, 856).
struct Geo64 {
    double t0, dt;
    __device__ double center(int k) const { return __dadd_rn(t0, __dmul_rn((double)k, dt)); }
    __device__ double start(int k) const {
        return __dadd_rn(t0, __dmul_rn(__dsub_rn((double)k, 0.5), dt));
    }
    __device__ double end(int k) const {
        return __dadd_rn(t0, __dmul_rn(__dadd_rn((double)k, 0.5), dt));
    }
    __device__ double per_dt(double x) const { return __ddiv_rn(x, dt); }
};
// One step of ChargedParticle::integrateFieldTrace (src/particle.cpp:786-865):
// the linear interpolant of the field over [ts1, ts2] is averaged over every
// bin it overlaps.  Decisions (window, case, indices) come from the point
// flags and bin indices; weights come from the coordinates u1, u2.
// Sink::add(k, f[6]) receives the bin contributions in increasing k.
template <class Ops, class Geo, class Sink>
__device__ __forceinline__ bool deposit_step(typename Ops::T u1, typename Ops::T u2, int idx1,
                                             int flags1, int idx2, int flags2,
                                             const typename Ops::T* f1,
                                             const typename Ops::T* f2, const Geo& geo, int nt,
                                             Sink& sink) {
    typedef typename Ops::T T;
    // (ts2 > tmin) && (ts1 < tmax)
    if ((flags2 & kLeTmin) || !(flags1 & kLtTmax)) return false;
    T dts = Ops::sub(u2, u1);
    T field[6];
    if (idx2 > nt) idx2 = nt;
    if (flags1 & kLeTmin) {
        // the step starts before the window: bins 0 .. idx2-1 fully covered
        for (int k = 0; k < idx2; k++) {
            T tc = geo.center(k);
            T w1 = Ops::div(Ops::sub(u2, tc), dts), w2 = Ops::div(Ops::sub(tc, u1), dts);
#pragma unroll
            for (int c = 0; c < 6; c++) field[c] = Ops::add(Ops::mul(f1[c], w1), Ops::mul(f2[c], w2));
            sink.add(k, field);
        }
        if (idx2 < nt) {
            T ts = geo.start(idx2);
            T w1 = Ops::div(Ops::sub(u2, ts), dts), w2 = Ops::div(Ops::sub(ts, u1), dts);
            T wb = geo.per_dt(Ops::sub(u2, ts));
#pragma unroll
            for (int c = 0; c < 6; c++) {
                T fs = Ops::add(Ops::mul(f1[c], w1), Ops::mul(f2[c], w2));
                field[c] = Ops::mul(Ops::mul(Ops::add(fs, f2[c]), (T)0.5), wb);
            }
            sink.add(idx2, field);
        }
    } else {
        if (idx1 == idx2) {
            // the step lies within one bin
            T wb = geo.per_dt(dts);
#pragma unroll
            for (int c = 0; c < 6; c++)
                field[c] = Ops::mul(Ops::mul(Ops::add(f1[c], f2[c]), (T)0.5), wb);
            sink.add(idx1, field);
        } else {
            // first partial bin
            T te = geo.end(idx1);
            T w1 = Ops::div(Ops::sub(u2, te), dts), w2 = Ops::div(Ops::sub(te, u1), dts);
            T wb = geo.per_dt(Ops::sub(te, u1));
#pragma unroll
            for (int c = 0; c < 6; c++) {
                T fe = Ops::add(Ops::mul(f1[c], w1), Ops::mul(f2[c], w2));
                field[c] = Ops::mul(Ops::mul(Ops::add(f1[c], fe), (T)0.5), wb);
            }
            sink.add(idx1, field);
            // fully covered bins
            for (int k = idx1 + 1; k < idx2; k++) {
                T tc = geo.center(k);
                T v1 = Ops::div(Ops::sub(u2, tc), dts), v2 = Ops::div(Ops::sub(tc, u1), dts);
#pragma unroll
                for (int c = 0; c < 6; c++)
                    field[c] = Ops::add(Ops::mul(f1[c], v1), Ops::mul(f2[c], v2));
                sink.add(k, field);
            }
            // last partial bin
            if (idx2 < nt) {
                T ts = geo.start(idx2);
                T x1 = Ops::div(Ops::sub(u2, ts), dts), x2 = Ops::div(Ops::sub(ts, u1), dts);
                T wl = geo.per_dt(Ops::sub(u2, ts));
#pragma unroll
                for (int c = 0; c < 6; c++) {
                    T fs = Ops::add(Ops::mul(f1[c], x1), Ops::mul(f2[c], x2));
                    field[c] = Ops::mul(Ops::mul(Ops::add(fs, f2[c]), (T)0.5), wl);
                }
                sink.add(idx2, field);
            }
        }
    }
    return true;
}

// Read-modify-write of one bin (6 components, 8- resp. 16-byte aligned).
__device__ __forceinline__ void add_row(float* row, const float* a) {
    float2* p = reinterpret_cast<float2*>(row);
    float2 v0 = p[0], v1 = p[1], v2 = p[2];
    v0.x += a[0];
    v0.y += a[1];
    v1.x += a[2];
    v1.y += a[3];
    v2.x += a[4];
    v2.y += a[5];
    p[0] = v0;
    p[1] = v1;
    p[2] = v2;
}
__device__ __forceinline__ void add_row(double* row, const double* a) {
    double2* p = reinterpret_cast<double2*>(row);
    double2 v0 = p[0], v1 = p[1], v2 = p[2];
    v0.x = __dadd_rn(v0.x, a[0]);
    v0.y = __dadd_rn(v0.y, a[1]);
    v1.x = __dadd_rn(v1.x, a[2]);
    v1.y = __dadd_rn(v1.y, a[3]);
    v2.x = __dadd_rn(v2.x, a[4]);
    v2.y = __dadd_rn(v2.y, a[5]);
    p[0] = v0;
    p[1] = v1;
    p[2] = v2;
}

// Accumulates the contributions of consecutive deposits into the open bin in
// registers and adds a finished bin into the pixel's partial trace.  Bins
// outside [0, nt) are the reference's range error: recorded and skipped.
template <class T, int STRIDE>
struct BinSink {
    T a[6];
    int open;
    int nt;
    T* row;  // this pixel's partial trace, [nt][STRIDE]
    unsigned int err;
    unsigned long long n_add;
    __device__ void init(T* r, int n) {
        row = r;
        nt = n;
        open = -1;
        err = 0;
        n_add = 0;
    }
    __device__ __forceinline__ void add(int k, const T* f) {
        if (k < 0 || k >= nt) {
            err |= 1u << TEUFEL_ERR_RANGE;
            return;
        }
        n_add++;
        if (k == open) {
#pragma unroll
            for (int c = 0; c < 6; c++) a[c] += f[c];
        } else {
            flush();
            open = k;
#pragma unroll
            for (int c = 0; c < 6; c++) a[c] = f[c];
        }
    }
    __device__ __forceinline__ void flush() {
        if (open < 0) return;
        add_row(row + (int64_t)open * STRIDE, a);
        open = -1;
    }
};

// Scale of the Lienard-Wiechert field of one particle:
// Charge*ElementaryCharge/(4.0*Pi*EpsNull), evaluated as src/particle.cpp:587
// from the charge in Coulomb (the product Charge*ElementaryCharge).
__device__ __forceinline__ double field_scale(double charge_C) {
    return __ddiv_rn(charge_C, __dmul_rn(__dmul_rn(4.0, kPi), kEps0));
}

__device__ __forceinline__ int warp_min(int v) { return __reduce_min_sync(0xffffffffu, v); }
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int warp_max(int v) { return __reduce_max_sync(0xffffffffu, v); }

// First particle whose segment range ends after global segment g.
__device__ __forceinline__ int particle_of_segment(const int64_t* seg_offsets, int n, int64_t g) {
    int lo = 0, hi = n;  // seg_offsets[n] = total
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (seg_offsets[mid + 1] > g) hi = mid; else lo = mid + 1;
    }
    return lo;
}

}  // namespace teufel
