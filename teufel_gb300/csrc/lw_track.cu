// lw_track.cu -- tracking on the device: the reference's Vay pusher
// (ChargedParticle::InitVay / StepVay, src/particle.cpp:407-512) writing the
// trajectory store directly, so trajectories never cross the host.
//
// The field is the reference's lattice of a planar undulator
// (PlanarUndulator::LocalField, src/undulator.cpp:107-125, placed at an
// origin as LocalizedField::Field does, src/fields.cpp:180-183) plus a
// homogeneous E/B field (HomogeneousField, src/fields.cpp:150-163), summed
// onto a zero field as Lattice::Field does.  One thread tracks one particle;
// every operation is an IEEE-rounded FP64 operation in the reference's order,
// so the trajectories agree with the reference's to the last bit except where
// CUDA's sin/cos/sinh/cosh and the host libm differ (an ulp).
#include <cuda_runtime.h>

#include "lw_common.cuh"

namespace teufel {

constexpr double kInvRestMass = 1.758820025e11;  // src/global.h:44

namespace {

struct V {
    double x, y, z;
};
__device__ __forceinline__ V add(V a, V b) {
    return V{__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z)};
}
__device__ __forceinline__ V sub(V a, V b) {
    return V{__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)};
}
__device__ __forceinline__ V mul(V a, double f) {
    return V{__dmul_rn(a.x, f), __dmul_rn(a.y, f), __dmul_rn(a.z, f)};
}
__device__ __forceinline__ V dvd(V a, double f) {
    return V{__ddiv_rn(a.x, f), __ddiv_rn(a.y, f), __ddiv_rn(a.z, f)};
}
__device__ __forceinline__ double abs2(V a) {
    return __dadd_rn(__dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)), __dmul_rn(a.z, a.z));
}
__device__ __forceinline__ double dot(V a, V b) {
    double t = __dmul_rn(a.x, b.x);
    t = __dadd_rn(t, __dmul_rn(a.y, b.y));
    return __dadd_rn(t, __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ V cross(V a, V b) {
    return V{__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)),
             __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
             __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x))};
}

// E and B of the lattice at X (time-independent elements)
__device__ void lattice_field(const TrackLattice& L, V X, V& E, V& B) {
    V e{0.0, 0.0, 0.0}, b{0.0, 0.0, 0.0};
    if (L.has_undulator) {
        const V x = sub(X, V{L.origin[0], L.origin[1], L.origin[2]});
        const double z1 = __ddiv_rn(-__dmul_rn((double)(L.n_periods + 1), L.lambda_u), 2.0);
        const double z2 = __ddiv_rn(__dmul_rn((double)(L.n_periods + 1), L.lambda_u), 2.0);
        V bu{0.0, 0.0, 0.0};
        if (z1 <= x.z && x.z < z2) {
            bu.y = __dmul_rn(__dmul_rn(L.b_peak, sin(__dmul_rn(L.kz, x.z))),
                             cosh(__dmul_rn(L.kz, x.y)));
            bu.z = __dmul_rn(__dmul_rn(L.b_peak, cos(__dmul_rn(L.kz, x.z))),
                             sinh(__dmul_rn(L.kz, x.y)));
            // one-period linear ramps at both ends
            if (x.z < __dadd_rn(z1, L.lambda_u))
                bu = mul(bu, __ddiv_rn(__dsub_rn(x.z, z1), L.lambda_u));
            if (__dsub_rn(z2, L.lambda_u) <= x.z)
                bu = mul(bu, __ddiv_rn(__dsub_rn(z2, x.z), L.lambda_u));
        }
        b = add(b, bu);
    }
    if (L.has_homogeneous) {
        e = add(e, V{L.e[0], L.e[1], L.e[2]});
        b = add(b, V{L.b[0], L.b[1], L.b[2]});
    }
    E = e;
    B = b;
}

struct Pusher {
    double dt, qm, qmt2, t;
    V X, P, A, p_i1;
    double gamma_i1;
};

// eqs. (11)-(12) of the Vay scheme (src/particle.cpp:428-437, 497-506)
__device__ __forceinline__ void second_half(Pusher& s, V E, V B) {
    const V p_prime = add(s.P, mul(dvd(E, kC), s.qmt2));
    const double gamma2_prime = __dadd_rn(abs2(p_prime), 1.0);
    const V tau = mul(B, s.qmt2);
    const double u_star = dot(p_prime, tau);
    const double tau2 = abs2(tau);
    const double sigma = __dsub_rn(gamma2_prime, tau2);
    s.gamma_i1 = __dsqrt_rn(__dmul_rn(
        0.5, __dadd_rn(sigma, __dsqrt_rn(__dadd_rn(
                                  __dmul_rn(sigma, sigma),
                                  __dmul_rn(4.0, __dadd_rn(tau2, __dmul_rn(u_star, u_star))))))));
    const V t = dvd(tau, s.gamma_i1);
    s.p_i1 = dvd(add(add(p_prime, mul(t, dot(p_prime, t))), cross(p_prime, t)),
                 __dadd_rn(1.0, abs2(t)));
}

__device__ __forceinline__ void store(const Pusher& s, double4_32a* tx, double4_32a* pp,
                                      double4_32a* aa) {
    *tx = make_double4_32a(s.t, s.X.x, s.X.y, s.X.z);
    *pp = make_double4_32a(s.P.x, s.P.y, s.P.z, 0.0);
    *aa = make_double4_32a(s.A.x, s.A.y, s.A.z, 0.0);
}

__global__ void vay_track_kernel(int n, const double* init, const double* charge_e,
                                 const double* mass, TrackLattice L, double tstep, int n_steps,
                                 double4_32a* tx, double4_32a* pp, double4_32a* aa,
                                 unsigned int* status) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const double* in = init + 7 * m;
    Pusher s;
    s.t = in[0];
    s.X = V{in[1], in[2], in[3]};
    s.P = V{in[4], in[5], in[6]};
    // InitVay (src/particle.cpp:407-438)
    s.dt = tstep;
    s.qm = __dmul_rn(__ddiv_rn(charge_e[m], mass[m]), kInvRestMass);
    s.qmt2 = __dmul_rn(__dmul_rn(s.qm, 0.5), s.dt);
    V E, B;
    lattice_field(L, s.X, E, B);
    second_half(s, E, B);
    {
        const double gamma_h = __dsqrt_rn(__dadd_rn(abs2(s.P), 1.0));
        const V beta_h = dvd(s.P, gamma_h);
        s.A = mul(add(cross(beta_h, B), dvd(E, kC)), s.qm);
    }
    const int64_t o = (int64_t)m * (n_steps + 1);
    store(s, tx + o, pp + o, aa + o);
    bool finite = isfinite(s.gamma_i1);
    // StepVay (src/particle.cpp:477-512)
    for (int k = 1; k <= n_steps; k++) {
        const V beta_i = dvd(s.p_i1, s.gamma_i1);
        s.t = __dadd_rn(s.t, s.dt);
        s.X = add(s.X, mul(mul(beta_i, kC), s.dt));
        lattice_field(L, s.X, E, B);
        s.P = add(s.p_i1, mul(add(dvd(E, kC), cross(beta_i, B)), s.qmt2));
        const double gamma_h = __dsqrt_rn(__dadd_rn(abs2(s.P), 1.0));
        const V beta_h = dvd(s.P, gamma_h);
        s.A = mul(add(cross(beta_h, B), dvd(E, kC)), s.qm);
        second_half(s, E, B);
        store(s, tx + o + k, pp + o + k, aa + o + k);
        finite = finite && isfinite(s.X.x + s.X.y + s.X.z + s.P.x + s.P.y + s.P.z);
    }
    if (!finite) atomicOr(status, 1u << TEUFEL_ERR_ARG);
}

}  // namespace

cudaError_t launch_vay_track(int n, const double* init, const double* charge_e,
                             const double* mass, const TrackLattice& L, double tstep, int n_steps,
                             double4_32a* tx, double4_32a* pp, double4_32a* aa,
                             unsigned int* status, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    vay_track_kernel<<<(n + 63) / 64, 64, 0, s>>>(n, init, charge_e, mass, L, tstep, n_steps, tx,
                                                  pp, aa, status);
    return cudaGetLastError();
}

}  // namespace teufel
