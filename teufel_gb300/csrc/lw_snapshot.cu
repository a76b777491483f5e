// lw_snapshot.cu -- the field at one observation time and place:
// ChargedParticle::RetardedField(double t, Vector X) (src/particle.cpp:612-769)
// summed over a particle set as Bunch::RetardedField does
// (src/bunch.cpp:729-737), for SnapshotObserver::integrate
// (src/snapshot.cpp:72-80).
//
// For every (observation point, particle) the emission point is found as the
// reference finds it: if the signal of the last trajectory point has not yet
// arrived there is no field; if not even the first point's has, the motion
// is extrapolated backwards from the first point at constant velocity
// (analytic light-cone intersection); otherwise the trajectory is bisected to
// the step whose signals bracket the observation time, and the emission
// point inside the step is refined by the secant method.  Everything is FP64
// with IEEE-rounded operations in the reference's order, so the bisection and
// refinement take the reference's decisions.  One thread per (point,
// particle chunk) accumulates its chunk in particle order; the chunks are
// added in order by a second kernel.
#include <cuda_runtime.h>

#include <algorithm>

#include "lw_common.cuh"

namespace teufel {

namespace {

struct d3 {
    double x, y, z;
};
__device__ __forceinline__ d3 sub(d3 a, d3 b) {
    return d3{__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)};
}
__device__ __forceinline__ d3 add(d3 a, d3 b) {
    return d3{__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z)};
}
__device__ __forceinline__ d3 mul(d3 a, double f) {
    return d3{__dmul_rn(a.x, f), __dmul_rn(a.y, f), __dmul_rn(a.z, f)};
}
__device__ __forceinline__ d3 dvd(d3 a, double f) {
    return d3{__ddiv_rn(a.x, f), __ddiv_rn(a.y, f), __ddiv_rn(a.z, f)};
}
// x*x + y*y + z*z left to right (src/vector.cpp:136-139)
__device__ __forceinline__ double abs2(d3 a) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)), __dmul_rn(a.z, a.z));
}
__device__ __forceinline__ double norm(d3 a) { return __dsqrt_rn(abs2(a)); }
// accumulated x, then y, then z (src/vector.cpp:157-164)
__device__ __forceinline__ double dot(d3 a, d3 b) {
    double t = __dmul_rn(a.x, b.x);
    t = __dadd_rn(t, __dmul_rn(a.y, b.y));
    return __dadd_rn(t, __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ d3 cross(d3 a, d3 b) {
    return d3{__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)),
              __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
              __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x))};
}
__device__ __forceinline__ d3 xyz(const double4_32a& v) { return d3{v.y, v.z, v.w}; }
__device__ __forceinline__ d3 vec(const double4_32a& v) { return d3{v.x, v.y, v.z}; }

// obs_time - (t + |o - x| / c): how early the signal of a point arrives
__device__ __forceinline__ double early(double obs_time, const double4_32a& tx, d3 o) {
    return __dsub_rn(obs_time, __dadd_rn(tx.x, __ddiv_rn(norm(sub(o, xyz(tx))), kC)));
}

// Adds the field of particle m at (obs_time, o) into acc.
__device__ void particle_field(const DevTraj& tr, int m, double obs_time, d3 o, double* acc) {
    const int64_t b = tr.offsets[m];
    const int64_t np = tr.offsets[m + 1] - b;
    const double4_32a* TX = tr.tx + b;
    const double4_32a* PP = tr.pp + b;
    const double4_32a* AA = tr.aa + b;
    int64_t i1 = 0, i2 = np - 1;
    double t1 = early(obs_time, TX[i1], o);
    double t2 = early(obs_time, TX[i2], o);
    if (!(t2 <= 0.0)) return;  // no signal has arrived yet (src/particle.cpp:631)
    d3 sx, beta, betap;
    double gamma2;
    if (t1 <= 0.0) {
        // back-extrapolation from the first point (src/particle.cpp:639-659)
        const d3 Rc = dvd(sub(o, xyz(TX[0])), kC);
        beta = vec(PP[0]);
        gamma2 = __dadd_rn(abs2(beta), 1.0);
        const double gamma = __dsqrt_rn(gamma2);
        beta = dvd(beta, gamma);
        const double t0 = obs_time;
        const double bR = dot(beta, Rc);
        const double bb = dot(beta, beta);
        const double RR = dot(Rc, Rc);
        const double a = __dsub_rn(t0, bR);
        const double disc =
            __dsub_rn(__dmul_rn(a, a), __dmul_rn(__dsub_rn(1.0, bb), __dsub_rn(__dmul_rn(t0, t0), RR)));
        const double st = __ddiv_rn(__dsub_rn(a, __dsqrt_rn(disc)), __dsub_rn(1.0, bb));
        sx = add(xyz(TX[0]), mul(mul(beta, kC), st));
        betap = d3{0.0, 0.0, 0.0};
    } else {
        // bisection to a single step (src/particle.cpp:666-685)
        while (i2 - i1 > 1) {
            const int64_t im = (i2 + i1) / 2;
            const double tm = early(obs_time, TX[im], o);
            if (tm > 0.0) {
                i1 = im;
                t1 = tm;
            } else {
                i2 = im;
                t2 = tm;
            }
        }
        double frac = __ddiv_rn(t1, __dsub_rn(t1, t2));
        // secant refinement (src/particle.cpp:693-733)
        const double tt1 = TX[i1].x, tt2 = TX[i2].x;
        const d3 X1 = xyz(TX[i1]), X2 = xyz(TX[i2]);
        auto source_t = [&](double f) {
            return __dadd_rn(__dmul_rn(tt1, __dsub_rn(1.0, f)), __dmul_rn(tt2, f));
        };
        auto source_x = [&](double f) { return add(mul(X1, __dsub_rn(1.0, f)), mul(X2, f)); };
        double st = source_t(frac);
        sx = source_x(frac);
        double R = norm(sub(o, sx));
        double dt = __dsub_rn(__dadd_rn(st, __ddiv_rn(R, kC)), obs_time);
        const double r1 = norm(sub(o, X1));
        const double r2 = norm(sub(o, X2));
        double dtdfrac = __dadd_rn(__dsub_rn(tt2, tt1), __ddiv_rn(__dsub_rn(r2, r1), kC));
        double dfrac = __ddiv_rn(dt, dtdfrac);
        int nref = 1;
        while (fabs(dfrac) > 1e-5 && nref < 10) {
            const double last = dt;
            frac = __dsub_rn(frac, dfrac);
            st = source_t(frac);
            sx = source_x(frac);
            R = norm(sub(o, sx));
            dt = __dsub_rn(__dadd_rn(st, __ddiv_rn(R, kC)), obs_time);
            dtdfrac = __ddiv_rn(-__dsub_rn(dt, last), dfrac);
            dfrac = __ddiv_rn(dt, dtdfrac);
            nref++;
        }
        frac = __dsub_rn(frac, dfrac);
        sx = source_x(frac);
        beta = add(mul(vec(PP[i1]), __dsub_rn(1.0, frac)), mul(vec(PP[i2]), frac));
        gamma2 = __dadd_rn(abs2(beta), 1.0);
        const double gamma = __dsqrt_rn(gamma2);
        beta = dvd(beta, gamma);
        betap = add(mul(vec(AA[i1]), __dsub_rn(1.0, frac)), mul(vec(AA[i2]), frac));
        betap = dvd(betap, gamma);
    }
    // the field of the source point (src/particle.cpp:750-766)
    const d3 rv = sub(o, sx);
    const double R = norm(rv);
    const double nn = norm(rv);
    const d3 n = d3{__ddiv_rn(rv.x, nn), __ddiv_rn(rv.y, nn), __ddiv_rn(rv.z, nn)};
    const double scale = field_scale(tr.charge[m]);
    const double k3 = pow(__dsub_rn(1.0, dot(beta, n)), 3.0);
    d3 E = dvd(sub(n, beta), __dmul_rn(__dmul_rn(__dmul_rn(R, R), k3), gamma2));
    const d3 acc_t = cross(n, cross(sub(n, beta), betap));
    E = add(E, dvd(acc_t, __dmul_rn(__dmul_rn(R, k3), kC)));
    E = mul(E, scale);
    const d3 B = dvd(cross(n, E), kC);
    acc[0] = __dadd_rn(acc[0], E.x);
    acc[1] = __dadd_rn(acc[1], E.y);
    acc[2] = __dadd_rn(acc[2], E.z);
    acc[3] = __dadd_rn(acc[3], B.x);
    acc[4] = __dadd_rn(acc[4], B.y);
    acc[5] = __dadd_rn(acc[5], B.z);
}

__global__ void retarded_field_kernel(DevTraj tr, double obs_time, int np, const double* pos,
                                      int chunk, double* partial) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const d3 o{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]};
    const int m0 = blockIdx.y * chunk;
    const int m1 = min(m0 + chunk, tr.n_particles);
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int m = m0; m < m1; m++) particle_field(tr, m, obs_time, o, acc);
    double* dst = partial + ((int64_t)blockIdx.y * np + p) * 6;
#pragma unroll
    for (int k = 0; k < 6; k++) dst[k] = acc[k];
}

__global__ void retarded_field_reduce_kernel(int np, int n_chunks, const double* partial,
                                             double* out) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)np * 6) return;
    double s = 0.0;
    for (int c = 0; c < n_chunks; c++) s = __dadd_rn(s, partial[(int64_t)c * np * 6 + e]);
    out[e] = s;
}

}  // namespace

int retarded_field_chunks(int np, int n_particles) {
    // about 600k threads in flight, at least 16 particles per chunk
    const int64_t want = (152LL * 4096 + np - 1) / std::max(np, 1);
    const int64_t most = (n_particles + 15) / 16;
    return (int)std::max<int64_t>(1, std::min<int64_t>(want, most));
}

cudaError_t launch_retarded_field(const DevTraj& tr, double obs_time, int np, const double* pos,
                                  int n_chunks, double* partial, double* out, cudaStream_t s) {
    if (np <= 0) return cudaSuccess;
    const int chunk = (tr.n_particles + n_chunks - 1) / n_chunks;
    dim3 grid((np + 127) / 128, n_chunks);
    retarded_field_kernel<<<grid, 128, 0, s>>>(tr, obs_time, np, pos, chunk, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int64_t n = (int64_t)np * 6;
    retarded_field_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(np, n_chunks, partial,
                                                                          out);
    return cudaGetLastError();
}

}  // namespace teufel
