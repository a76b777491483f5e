// trajgen.cpp -- synthetic trajectory source for the field integration.
//
// The field-integration path consumes tracked trajectories (t, x, beta*gamma,
// d(beta*gamma)/dt per point).  TEUFEL produces them with its Vay pusher; the
// pusher itself is not part of the accelerated path, so this file provides a
// host-side trajectory source with the same arithmetic, used to feed
// identical seeded inputs to every implementation of the field integration:
//
//   ChargedParticle::InitVay / StepVay      src/particle.cpp:407-512
//   ChargedParticle::initTrajectory         src/particle.cpp:345-360
//   PlanarUndulator::LocalField             src/undulator.cpp:107-125
//   LocalizedField::Field (origin shift)    src/fields.cpp:180-183
//   HomogeneousField::Field                 src/fields.cpp:150-163
//
// Operations are written in the reference's evaluation order and the file is
// compiled with -ffp-contract=off, so on one machine the trajectories are
// bit-identical to the ones the reference's own pusher produces (checked in
// tests/test_oracle_pusher.py and tests/test_oracle_vs_ref.py against fixtures
// made by the compiled reference).
//
// The bunch sampler (splitmix64 + Box-Muller) is this project's own: the
// reference seeds from std::random_device (src/bunch.cpp:40-41), which is not
// reproducible, so every path here draws from one seeded stream instead.
#include <cmath>
#include <cstdint>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kE = 1.6021766208e-19;      // src/global.h:36
constexpr double kMeC2 = 0.5109989461e6;     // src/global.h:37 [eV]
constexpr double kC = 2.99792458e8;          // src/global.h:38
constexpr double kPi = 3.1415926535897932384626433832795029;
constexpr double kInvRestMass = 1.758820025e11;  // src/global.h:43

struct V3 {
    double x, y, z;
};
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 mul(V3 a, double f) { return {a.x * f, a.y * f, a.z * f}; }
inline V3 dvd(V3 a, double f) { return {a.x / f, a.y / f, a.z / f}; }
inline double abs2(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline double dot(V3 a, V3 b) {
    double t = a.x * b.x;
    t += a.y * b.y;
    t += a.z * b.z;
    return t;
}
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Lattice description: a planar undulator centred at `origin` plus an
// optional homogeneous field (both may be present; fields add).
struct Lattice {
    int has_und;
    double b_peak, lambda_u, kz;
    int n_periods;
    V3 origin;
    int has_hom;
    V3 hom_e, hom_b;
};

inline void und_local(const Lattice& L, V3 X, V3* B) {
    // PlanarUndulator::LocalField: field in (z1, z2) with one-period linear ramps
    double z1 = -(L.n_periods + 1) * L.lambda_u / 2.0;
    double z2 = (L.n_periods + 1) * L.lambda_u / 2.0;
    V3 b = {0.0, 0.0, 0.0};
    if (z1 <= X.z && X.z < z2) {
        b.x = 0.0;
        b.y = L.b_peak * std::sin(L.kz * X.z) * std::cosh(L.kz * X.y);
        b.z = L.b_peak * std::cos(L.kz * X.z) * std::sinh(L.kz * X.y);
        if (X.z < z1 + L.lambda_u) b = mul(b, (X.z - z1) / L.lambda_u);
        if (z2 - L.lambda_u <= X.z) b = mul(b, (z2 - X.z) / L.lambda_u);
    }
    *B = b;
}

inline void lattice_field(const Lattice& L, V3 X, V3* E, V3* B) {
    // Lattice::Field sums the elements onto a zero field
    V3 e = {0.0, 0.0, 0.0}, b = {0.0, 0.0, 0.0};
    if (L.has_und) {
        V3 bu;
        und_local(L, sub(X, L.origin), &bu);
        b = add(b, bu);
    }
    if (L.has_hom) {
        e = add(e, L.hom_e);
        b = add(b, L.hom_b);
    }
    *E = e;
    *B = b;
}

// State carried between Vay steps (the reference's ChargedParticle members)
struct Pusher {
    double dt, qm, qmt2;
    double t;
    V3 X, P, A, p_i1;
    double gamma_i1;
};

inline void vay_second_half(Pusher& s, V3 E, V3 B) {
    // eqs. (11)-(12) of the Vay scheme as written in src/particle.cpp:430-437
    V3 p_prime = add(s.P, mul(dvd(E, kC), s.qmt2));
    double gamma2_prime = abs2(p_prime) + 1.0;
    V3 tau = mul(B, s.qmt2);
    double u_star = dot(p_prime, tau);
    double tau2 = abs2(tau);
    double sigma = gamma2_prime - tau2;
    s.gamma_i1 = std::sqrt(0.5 * (sigma + std::sqrt(sigma * sigma + 4.0 * (tau2 + u_star * u_star))));
    V3 t = dvd(tau, s.gamma_i1);
    s.p_i1 = dvd(add(add(p_prime, mul(t, dot(p_prime, t))), cross(p_prime, t)), (1 + abs2(t)));
}

inline void vay_init(Pusher& s, const Lattice& L, double charge, double mass, double tstep) {
    s.dt = tstep;
    s.qm = charge / mass * kInvRestMass;
    s.qmt2 = s.qm * 0.5 * s.dt;
    V3 E, B;
    lattice_field(L, s.X, &E, &B);
    vay_second_half(s, E, B);
    double gamma_h = std::sqrt(abs2(s.P) + 1.0);
    V3 beta_h = dvd(s.P, gamma_h);
    s.A = mul(add(cross(beta_h, B), dvd(E, kC)), s.qm);
}

inline void vay_step(Pusher& s, const Lattice& L) {
    V3 p_i = s.p_i1;
    V3 beta_i = dvd(p_i, s.gamma_i1);
    s.t += s.dt;
    s.X = add(s.X, mul(mul(beta_i, kC), s.dt));
    V3 E, B;
    lattice_field(L, s.X, &E, &B);
    s.P = add(s.p_i1, mul(add(dvd(E, kC), cross(beta_i, B)), s.qmt2));
    double gamma_h = std::sqrt(abs2(s.P) + 1.0);
    V3 beta_h = dvd(s.P, gamma_h);
    s.A = mul(add(cross(beta_h, B), dvd(E, kC)), s.qm);
    vay_second_half(s, E, B);
}

// splitmix64: a counter-based generator, so particle m's draws do not depend
// on how many threads generate the bunch
inline uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
inline double uniform01(uint64_t& s) {  // (0, 1]
    return (double)((splitmix64(s) >> 11) + 1) * (1.0 / 9007199254740992.0);
}
inline void gauss2(uint64_t& s, double* g0, double* g1) {
    double u1 = uniform01(s), u2 = uniform01(s);
    double r = std::sqrt(-2.0 * std::log(u1));
    *g0 = r * std::cos(2.0 * kPi * u2);
    *g1 = r * std::sin(2.0 * kPi * u2);
}

}  // namespace

extern "C" {

// Peak field of a planar undulator with deflection parameter K:
// B0 = 2 pi m c K / (e lambda_u) = 2 pi (m c^2 / e) K / (c lambda_u).
double tg_undulator_b0(double K, double lambda_u) {
    return 2.0 * kPi * kMeC2 * K / (kC * lambda_u);
}

// Track n_part particles for n_steps Vay steps each (n_steps+1 stored points,
// the first one being the initial condition with its acceleration replaced by
// the one InitVay computes).
//   init[n_part][7]: t, x, y, z, px, py, pz   (p = beta*gamma)
//   lat[16]: has_und, b_peak, lambda_u, n_periods, ox, oy, oz,
//            has_hom, Ex, Ey, Ez, Bx, By, Bz, (unused) x2
//   out_t[n_part*(n_steps+1)], out_x/out_p/out_a[...][3]
int tg_track(int64_t n_part, const double* init, double charge, double mass, const double* lat,
             double tstep, int64_t n_steps, double* out_t, double* out_x, double* out_p,
             double* out_a, int nthreads) {
    if (n_part < 0 || n_steps < 0 || !(tstep > 0.0)) return 1;
    Lattice L;
    L.has_und = lat[0] != 0.0;
    L.b_peak = lat[1];
    L.lambda_u = lat[2];
    L.n_periods = (int)lat[3];
    L.origin = {lat[4], lat[5], lat[6]};
    L.kz = 2.0 * kPi / L.lambda_u;
    L.has_hom = lat[7] != 0.0;
    L.hom_e = {lat[8], lat[9], lat[10]};
    L.hom_b = {lat[11], lat[12], lat[13]};
    const int64_t np = n_steps + 1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t m = 0; m < n_part; m++) {
        const double* in = init + 7 * m;
        Pusher s;
        s.t = in[0];
        s.X = {in[1], in[2], in[3]};
        s.P = {in[4], in[5], in[6]};
        s.A = {0.0, 0.0, 0.0};
        vay_init(s, L, charge, mass, tstep);
        double* ot = out_t + np * m;
        double* ox = out_x + 3 * np * m;
        double* op = out_p + 3 * np * m;
        double* oa = out_a + 3 * np * m;
        ot[0] = s.t;
        std::memcpy(ox, &s.X, 24);
        std::memcpy(op, &s.P, 24);
        std::memcpy(oa, &s.A, 24);
        for (int64_t k = 1; k < np; k++) {
            vay_step(s, L);
            ot[k] = s.t;
            std::memcpy(ox + 3 * k, &s.X, 24);
            std::memcpy(op + 3 * k, &s.P, 24);
            std::memcpy(oa + 3 * k, &s.A, 24);
        }
    }
    return 0;
}

// Seeded 6-D Gaussian bunch with no correlations.  Particle m draws from its
// own stream seeded by (seed, m), so any subset of a bunch can be generated
// on its own and agrees with the full bunch.
//   out[n][7]: t(=0), x, y, z, px, py, pz with pz from the drawn gamma.
void tg_gaussian_bunch(int64_t first, int64_t n, uint64_t seed, double sx, double sy, double sz,
                       double spx, double spy, double gamma0, double sgamma, double z0,
                       double* out) {
    for (int64_t i = 0; i < n; i++) {
        uint64_t st = seed * 0x9E3779B97F4A7C15ULL ^ (uint64_t)(first + i) * 0xD1B54A32D192ED03ULL;
        splitmix64(st);
        double g[6];
        gauss2(st, &g[0], &g[1]);
        gauss2(st, &g[2], &g[3]);
        gauss2(st, &g[4], &g[5]);
        double x = sx * g[0], y = sy * g[1], z = z0 + sz * g[2];
        double px = spx * g[3], py = spy * g[4];
        double gamma = gamma0 + sgamma * g[5];
        double pz2 = gamma * gamma - 1.0 - px * px - py * py;
        double pz = pz2 > 0.0 ? std::sqrt(pz2) : 0.0;
        double* o = out + 7 * i;
        o[0] = 0.0;
        o[1] = x;
        o[2] = y;
        o[3] = z;
        o[4] = px;
        o[5] = py;
        o[6] = pz;
    }
}

// Uniform draws for batch parameters (seeded, reproducible)
void tg_uniform(uint64_t seed, int64_t n, double lo, double hi, double* out) {
    uint64_t st = seed;
    for (int64_t i = 0; i < n; i++) out[i] = lo + (hi - lo) * (uniform01(st) - 0.0);
}

}  // extern "C"
