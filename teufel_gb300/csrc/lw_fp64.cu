// lw_fp64.cu -- the plain FP64 field-integration kernel.
//
// Same work decomposition as the split-precision kernel (one thread per
// pixel, particle-range slots, bisection for the in-window steps, each
// trajectory point evaluated once), but every quantity is computed in FP64
// with IEEE-rounded operations in the order of the reference:
//   RetardedTime   src/particle.cpp:560-568
//   RetardedField  src/particle.cpp:570-596
//   deposit        src/particle.cpp:786-865
// It is the GPU comparison path for the split-precision kernel and the
// oracle the split path's traces are measured against on the device.
#include <cuda_runtime.h>

#include "lw_common.cuh"

namespace teufel {

namespace {
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
}  // namespace

// ChargedParticle::RetardedField(int, Vector), src/particle.cpp:570-596.
__device__ __forceinline__ void exact_field(const double4_32a tx, const double4_32a p, const double4_32a a,
                                            double scale, const double3 obs, double f[6]) {
    double bg2 = dadd(dadd(dmul(p.x, p.x), dmul(p.y, p.y)), dmul(p.z, p.z));
    double gamma2 = dadd(bg2, 1.0);
    double gamma = __dsqrt_rn(gamma2);
    double bx = ddiv(p.x, gamma), by = ddiv(p.y, gamma), bz = ddiv(p.z, gamma);
    double ax = ddiv(a.x, gamma), ay = ddiv(a.y, gamma), az = ddiv(a.z, gamma);
    double rx = dsub(obs.x, tx.y), ry = dsub(obs.y, tx.z), rz = dsub(obs.z, tx.w);
    double R = __dsqrt_rn(dadd(dadd(dmul(rx, rx), dmul(ry, ry)), dmul(rz, rz)));
    double nx = ddiv(rx, R), ny = ddiv(ry, R), nz = ddiv(rz, R);
    double bn = dmul(bx, nx);
    bn = dadd(bn, dmul(by, ny));
    bn = dadd(bn, dmul(bz, nz));
    double k3 = pow(dsub(1.0, bn), 3.0);
    double mx = dsub(nx, bx), my = dsub(ny, by), mz = dsub(nz, bz);
    double d1 = dmul(dmul(dmul(R, R), k3), gamma2);
    double Ex = ddiv(mx, d1), Ey = ddiv(my, d1), Ez = ddiv(mz, d1);
    // cross(N - beta, beta')
    double cx = dsub(dmul(my, az), dmul(mz, ay));
    double cy = dsub(dmul(mz, ax), dmul(mx, az));
    double cz = dsub(dmul(mx, ay), dmul(my, ax));
    // cross(N, that)
    double qx = dsub(dmul(ny, cz), dmul(nz, cy));
    double qy = dsub(dmul(nz, cx), dmul(nx, cz));
    double qz = dsub(dmul(nx, cy), dmul(ny, cx));
    double d2 = dmul(dmul(R, k3), kC);
    Ex = dadd(Ex, ddiv(qx, d2));
    Ey = dadd(Ey, ddiv(qy, d2));
    Ez = dadd(Ez, ddiv(qz, d2));
    Ex = dmul(Ex, scale);
    Ey = dmul(Ey, scale);
    Ez = dmul(Ez, scale);
    f[0] = Ex;
    f[1] = Ey;
    f[2] = Ez;
    f[3] = ddiv(dsub(dmul(ny, Ez), dmul(nz, Ey)), kC);
    f[4] = ddiv(dsub(dmul(nz, Ex), dmul(nx, Ez)), kC);
    f[5] = ddiv(dsub(dmul(nx, Ey), dmul(ny, Ex)), kC);
}

struct Point64 {
    double ts;
    int idx, flags;
    double f[6];
};

__device__ __forceinline__ void eval_point64(Point64& S, const DevTraj& tr, int64_t i,
                                             double scale, const double3 P, const Window& w) {
    double4_32a tx = tr.tx[i];
    S.ts = exact_retarded_time(tx, P);
    S.idx = exact_bin(S.ts, w);
    S.flags = exact_flags(S.ts, w);
    exact_field(tx, tr.pp[i], tr.aa[i], scale, P, S.f);
}

__global__ void __launch_bounds__(128)
    lw_fp64_kernel(DevTraj tr, DevScreen sc, DevWork wk) {
    const int slot = blockIdx.y;
    const int pix = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = pix < sc.np;
    const int pc = active ? pix : sc.np - 1;
    const double3 P = make_double3(sc.pix_pos[3 * pc], sc.pix_pos[3 * pc + 1],
                                   sc.pix_pos[3 * pc + 2]);
    const Window w = make_window(sc.pix_t0[pc], sc.dt, sc.nt);
    const Geo64 geo{w.t0, w.dt};
    BinSink<double, 6> sink;
    sink.init(static_cast<double*>(wk.scratch) + (int64_t)slot * wk.slot_stride +
                  (int64_t)pc * sc.nt * 6,
              sc.nt);
    const int64_t g0 = wk.slot_seg[slot], g1 = wk.slot_seg[slot + 1];
    int m = g0 < g1 ? particle_of_segment(tr.seg_offsets, tr.n_particles, g0) : tr.n_particles;
    unsigned long long inwin = 0, nev = 0;
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
        if (st_lo >= st_hi || !active) continue;
        int first = st_lo, last = st_hi - 1;
        if (tr.vhat[m].w > 0.0)
            inwindow_steps(tr.tx + po, st_lo, st_hi, P, w, tr.vhat[m].w, &first, &last);
        if (last < first) continue;
        const double scale = field_scale(tr.charge[m]);
        Point64 p1, p2;
        nev += (unsigned long long)(last - first + 2);
        eval_point64(p1, tr, po + first, scale, P, w);
        for (int s = first; s <= last; ++s) {
            eval_point64(p2, tr, po + s + 1, scale, P, w);
            if (deposit_step<Ops64>(p1.ts, p2.ts, p1.idx, p1.flags, p2.idx, p2.flags, p1.f,
                                    p2.f, geo, sc.nt, sink))
                inwin++;
            p1 = p2;
        }
    }
    sink.flush();
    if (sink.err) atomicOr(wk.status, sink.err);
    inwin = warp_sum_u64(inwin);
    unsigned long long nadd = warp_sum_u64(sink.n_add);
    nev = warp_sum_u64(nev);
    if ((threadIdx.x & 31) == 0 && wk.counters) {
        if (inwin) atomicAdd(wk.counters, inwin);
        if (nadd) atomicAdd(wk.counters + 2, nadd);
        if (nev) atomicAdd(wk.counters + 3, nev);
    }
}

cudaError_t launch_fp64(const DevTraj& tr, const DevScreen& sc, const DevWork& w, int threads,
                        cudaStream_t s) {
    if (threads != 128) threads = 128;
    dim3 grid((sc.np + threads - 1) / threads, w.n_slots);
    lw_fp64_kernel<<<grid, threads, 0, s>>>(tr, sc, w);
    return cudaGetLastError();
}

}  // namespace teufel
