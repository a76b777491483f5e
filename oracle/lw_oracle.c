/*
 * lw_oracle.c -- CPU oracle for the Lienard-Wiechert field-trace integration.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is loaded by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and
 * by nothing on the product path.  The product (teufel_gb300/) never links,
 * imports or calls it.
 *
 * It restates, in plain C with IEEE double arithmetic and no FMA contraction
 * (build with -ffp-contract=off), the algorithm of TEUFEL 0.11.1:
 *
 *   ChargedParticle::RetardedTime(int, Vector)      src/particle.cpp:560-568
 *   ChargedParticle::RetardedField(int, Vector)     src/particle.cpp:570-596
 *   ChargedParticle::integrateFieldTrace(...)       src/particle.cpp:771-867
 *   Bunch::integrateFieldTrace (particle order)     src/bunch.cpp:739-745
 *   FieldTrace::add range check                     src/fieldtrace.cpp:185-190
 *   Vector::norm / dot / cross evaluation order     src/vector.cpp:136-170
 *   MeshedScreen<...>::integrate pixel loop         src/mesh.cpp:289-316
 *   ScreenObserver<...>::CellPosition/CellTimeZero  src/screen.cpp:97-110
 *
 * Every floating-point operation is written in the order the reference
 * evaluates it, so that retarded times and bin indices are bit-identical to
 * the reference on the same machine.  Physical constants follow
 * src/global.h:36-44.
 *
 * Parity pins: tests/test_oracle_kat.py checks the deposit against the
 * reference's own known-answer test (tests/teufel.integrate_field.cpp:98-189)
 * and tests/test_oracle_vs_ref.py checks whole traces against fixtures that
 * tests/golden/make_golden.py produced by running the reference's compiled
 * particle.cpp (oracle/_ref) on the same trajectories.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/global.h:36-44 */
#define LWO_E_CHARGE 1.6021766208e-19
#define LWO_C 2.99792458e8
#define LWO_PI 3.1415926535897932384626433832795029
#define LWO_EPS0 8.854187817e-12

/* status codes shared with include/teufel_cuda.h */
#define LWO_OK 0
#define LWO_ERR_RANGE 4

typedef struct { double x, y, z; } v3;

static v3 v3_sub(v3 a, v3 b) { v3 r; r.x = a.x - b.x; r.y = a.y - b.y; r.z = a.z - b.z; return r; }
static v3 v3_add(v3 a, v3 b) { v3 r; r.x = a.x + b.x; r.y = a.y + b.y; r.z = a.z + b.z; return r; }
static v3 v3_mul(v3 a, double f) { v3 r; r.x = a.x * f; r.y = a.y * f; r.z = a.z * f; return r; }
static v3 v3_div(v3 a, double f) { v3 r; r.x = a.x / f; r.y = a.y / f; r.z = a.z / f; return r; }
/* sqrt(x*x+y*y+z*z), left to right (src/vector.cpp:136-139) */
static double v3_norm(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static double v3_abs2(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
/* accumulate x, then y, then z (src/vector.cpp:157-164) */
static double v3_dot(v3 a, v3 b) { double t = a.x * b.x; t += a.y * b.y; t += a.z * b.z; return t; }
static v3 v3_cross(v3 a, v3 b)
{
    v3 r;
    r.x = a.y * b.z - a.z * b.y;
    r.y = a.z * b.x - a.x * b.z;
    r.z = a.x * b.y - a.y * b.x;
    return r;
}

/* six field components Ex,Ey,Ez,Bx,By,Bz -- the ElMagField layout */
typedef struct { double c[6]; } f6;

static f6 f6_lin(f6 a, double wa, f6 b, double wb)
{
    /* a*wa + b*wb, each product rounded separately (ElMagField ops) */
    f6 r;
    for (int k = 0; k < 6; k++) r.c[k] = a.c[k] * wa + b.c[k] * wb;
    return r;
}

static int trace_add(double *trace, int64_t nots, int64_t idx, f6 f, int *err)
{
    /* FieldTrace::add throws when the index is out of range (src/fieldtrace.cpp:185-190);
       here the first such event sets the error flag and the deposit is skipped. */
    if (idx < 0 || idx >= nots) { *err = LWO_ERR_RANGE; return 0; }
    double *b = trace + 6 * idx;
    for (int k = 0; k < 6; k++) b[k] += f.c[k];
    return 1;
}

/* ts = t + |obs - x| / c  (src/particle.cpp:560-568) */
double lwo_retarded_time(double t, const double *x, const double *obs)
{
    v3 o = {obs[0], obs[1], obs[2]};
    v3 p = {x[0], x[1], x[2]};
    v3 r = v3_sub(o, p);
    double R = v3_norm(r);
    return t + R / LWO_C;
}

/* Lienard-Wiechert field of one trajectory point (src/particle.cpp:570-596).
   bg = beta*gamma, a = d(beta*gamma)/dt, charge in units of e. */
void lwo_retarded_field(const double *x, const double *bg, const double *a,
                        double charge, const double *obs, double *out6)
{
    v3 X = {x[0], x[1], x[2]};
    v3 beta = {bg[0], bg[1], bg[2]};
    v3 betap = {a[0], a[1], a[2]};
    double bg2 = v3_abs2(beta);
    double gamma2 = bg2 + 1.0;
    double gamma = sqrt(gamma2);
    beta = v3_div(beta, gamma);
    betap = v3_div(betap, gamma);
    v3 o = {obs[0], obs[1], obs[2]};
    v3 rv = v3_sub(o, X);
    double R = v3_norm(rv);
    v3 n = rv;
    double nn = v3_norm(n);
    n.x /= nn; n.y /= nn; n.z /= nn;
    double scale = charge * LWO_E_CHARGE / (4.0 * LWO_PI * LWO_EPS0);
    double k3 = pow(1.0 - v3_dot(beta, n), 3.0);
    v3 nmb = v3_sub(n, beta);
    v3 E = v3_div(nmb, R * R * k3 * gamma2);
    v3 acc = v3_cross(n, v3_cross(v3_sub(n, beta), betap));
    E = v3_add(E, v3_div(acc, R * k3 * LWO_C));
    E = v3_mul(E, scale);
    v3 B = v3_div(v3_cross(n, E), LWO_C);
    out6[0] = E.x; out6[1] = E.y; out6[2] = E.z;
    out6[3] = B.x; out6[4] = B.y; out6[5] = B.z;
}

/* The interval-overlap deposit of one trajectory step [ts1, ts2] carrying the
   fields f1 (at ts1) and f2 (at ts2) into a trace of nots bins of width dt
   centred on t0 + k*dt (src/particle.cpp:786-865, one loop iteration).
   Returns 1 if the step touched the trace window. */
int lwo_deposit_step(double ts1, double ts2, const double *f1p, const double *f2p,
                     double t0, double dt, int64_t nots, double *trace, int *err)
{
    double tmin = t0 - dt * 0.5;
    double tmax = t0 + dt * ((double)nots - 0.5);
    double dts = ts2 - ts1;
    if (!((ts2 > tmin) && (ts1 < tmax))) return 0;
    f6 f1, f2, field;
    memcpy(f1.c, f1p, sizeof f1.c);
    memcpy(f2.c, f2p, sizeof f2.c);
    if (ts1 <= tmin) {
        /* the step starts before the window: fully covered bins 0..idx2-1,
           then the partially covered bin idx2 */
        int64_t idx2 = (int64_t)round((ts2 - t0) / dt);
        if (idx2 > nots) idx2 = nots;
        for (int64_t idx = 0; idx < idx2; idx++) {
            double tc = t0 + idx * dt;
            field = f6_lin(f1, (ts2 - tc) / dts, f2, (tc - ts1) / dts);
            trace_add(trace, nots, idx, field, err);
        }
        if (idx2 < nots) {
            double ts = t0 + (idx2 - 0.5) * dt;
            f6 fs = f6_lin(f1, (ts2 - ts) / dts, f2, (ts - ts1) / dts);
            for (int k = 0; k < 6; k++) field.c[k] = (fs.c[k] + f2.c[k]) * 0.5 * ((ts2 - ts) / dt);
            trace_add(trace, nots, idx2, field, err);
        }
    } else {
        int64_t idx1 = (int64_t)round((ts1 - t0) / dt);
        int64_t idx2 = (int64_t)round((ts2 - t0) / dt);
        if (idx2 > nots) idx2 = nots;
        if (idx1 == idx2) {
            for (int k = 0; k < 6; k++) field.c[k] = (f1.c[k] + f2.c[k]) * 0.5 * (dts / dt);
            trace_add(trace, nots, idx1, field, err);
        } else {
            double te = t0 + (idx1 + 0.5) * dt;
            f6 fe = f6_lin(f1, (ts2 - te) / dts, f2, (te - ts1) / dts);
            for (int k = 0; k < 6; k++) field.c[k] = (f1.c[k] + fe.c[k]) * 0.5 * ((te - ts1) / dt);
            trace_add(trace, nots, idx1, field, err);
            for (int64_t idx = idx1 + 1; idx < idx2; idx++) {
                double tc = t0 + idx * dt;
                field = f6_lin(f1, (ts2 - tc) / dts, f2, (tc - ts1) / dts);
                trace_add(trace, nots, idx, field, err);
            }
            if (idx2 < nots) {
                double ts = t0 + (idx2 - 0.5) * dt;
                f6 fs = f6_lin(f1, (ts2 - ts) / dts, f2, (ts - ts1) / dts);
                for (int k = 0; k < 6; k++) field.c[k] = (fs.c[k] + f2.c[k]) * 0.5 * ((ts2 - ts) / dt);
                trace_add(trace, nots, idx2, field, err);
            }
        }
    }
    return 1;
}

/* One particle onto one observation point (src/particle.cpp:771-867).
   t[np], x/bg/a[np][3].  Adds into trace[nots][6].  Returns the number of
   steps that touched the window. */
int64_t lwo_integrate_particle(int64_t np, const double *t, const double *x,
                               const double *bg, const double *a, double charge,
                               const double *obs, double t0, double dt, int64_t nots,
                               double *trace, int *err)
{
    if (nots < 2) return 0;
    if (np < 2) return 0;
    double tmin = t0 - dt * 0.5;
    double tmax = t0 + dt * ((double)nots - 0.5);
    int64_t touched = 0;
    /* the reference evaluates both end points of every step; the values
       are the same numbers, so each point is computed once and reused */
    double ts1 = lwo_retarded_time(t[0], x, obs);
    double f1[6], f2[6];
    int have_f1 = 0;
    for (int64_t step = 0; step < np - 1; step++) {
        double ts2 = lwo_retarded_time(t[step + 1], x + 3 * (step + 1), obs);
        if ((ts2 > tmin) && (ts1 < tmax)) {
            if (!have_f1)
                lwo_retarded_field(x + 3 * step, bg + 3 * step, a + 3 * step, charge, obs, f1);
            lwo_retarded_field(x + 3 * (step + 1), bg + 3 * (step + 1), a + 3 * (step + 1), charge, obs, f2);
            touched += lwo_deposit_step(ts1, ts2, f1, f2, t0, dt, nots, trace, err);
            memcpy(f1, f2, sizeof f1);
            have_f1 = 1;
        } else {
            have_f1 = 0;
        }
        ts1 = ts2;
    }
    return touched;
}

/* A set of particles (a Bunch, src/bunch.cpp:739-745) onto many observation
   points, OpenMP over points as src/mesh.cpp:296 does.  offsets[n_part+1]
   indexes the concatenated point arrays.  out[n_pix][nots][6] is added into.
   Returns the first error code met (0 if none). */
int lwo_integrate_screen(int64_t n_part, const int64_t *offsets, const double *charge,
                         const double *t, const double *x, const double *bg, const double *a,
                         int64_t n_pix, const double *pix_pos, const double *pix_t0,
                         double dt, int64_t nots, double *out, int nthreads,
                         int64_t *touched_out)
{
    int err_all = LWO_OK;
    int64_t touched = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(static) reduction(+ : touched)
    for (int64_t ip = 0; ip < n_pix; ip++) {
        int err = LWO_OK;
        for (int64_t m = 0; m < n_part; m++) {
            int64_t o = offsets[m];
            touched += lwo_integrate_particle(offsets[m + 1] - o, t + o, x + 3 * o, bg + 3 * o,
                                              a + 3 * o, charge[m], pix_pos + 3 * ip, pix_t0[ip],
                                              dt, nots, out + 6 * nots * ip, &err);
        }
        if (err != LWO_OK) {
#pragma omp critical
            { if (err_all == LWO_OK) err_all = err; }
        }
    }
    if (touched_out) *touched_out = touched;
    return err_all;
}

/* The same integration with arrival times evaluated in long double (64-bit
   significand on x86-64, 113 bits on aarch64) and deposited in bin units:
   an accuracy reference for cases where the FP64 flight time's own rounding
   matters (attosecond bins 30 m from the source).  Fields are the FP64
   restatement.  Bins and weights follow lwo_deposit_step with t0 = 0, dt = 1
   on u = (ts - t0)/dt. */
int lwo_integrate_screen_ext(int64_t n_part, const int64_t *offsets, const double *charge,
                             const double *t, const double *x, const double *bg, const double *a,
                             int64_t n_pix, const double *pix_pos, const double *pix_t0,
                             double dt, int64_t nots, double *out, int nthreads)
{
    int err_all = LWO_OK;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(static)
    for (int64_t ip = 0; ip < n_pix; ip++) {
        int err = LWO_OK;
        const double *obs = pix_pos + 3 * ip;
        double *trace = out + 6 * nots * ip;
        for (int64_t m = 0; m < n_part && nots >= 2; m++) {
            int64_t o = offsets[m], np = offsets[m + 1] - o;
            if (np < 2) continue;
            double u1 = 0.0, f1[6], f2[6];
            for (int64_t i = 0; i < np; i++) {
                const double *xi = x + 3 * (o + i);
                long double rx = (long double)obs[0] - xi[0];
                long double ry = (long double)obs[1] - xi[1];
                long double rz = (long double)obs[2] - xi[2];
                long double R = sqrtl(rx * rx + ry * ry + rz * rz);
                long double ts = (long double)t[o + i] + R / (long double)LWO_C;
                double u2 = (double)((ts - (long double)pix_t0[ip]) / (long double)dt);
                lwo_retarded_field(xi, bg + 3 * (o + i), a + 3 * (o + i), charge[m], obs, f2);
                if (i > 0) lwo_deposit_step(u1, u2, f1, f2, 0.0, 1.0, nots, trace, &err);
                u1 = u2;
                memcpy(f1, f2, sizeof f1);
            }
        }
        if (err != LWO_OK) {
#pragma omp critical
            { if (err_all == LWO_OK) err_all = err; }
        }
    }
    return err_all;
}

/* Deposit-only entry for the known-answer test: particle m has np[m] points
   with given arrival times ts and fields f[6] (what the reference's KAT
   injects by overriding RetardedTime/RetardedField). */
int lwo_deposit_injected(int64_t n_part, const int64_t *offsets, const double *ts,
                         const double *f, double t0, double dt, int64_t nots, double *trace)
{
    int err = LWO_OK;
    if (nots < 2) return err;
    for (int64_t m = 0; m < n_part; m++) {
        int64_t o = offsets[m], np = offsets[m + 1] - o;
        if (np < 2) continue;
        for (int64_t s = 0; s < np - 1; s++)
            lwo_deposit_step(ts[o + s], ts[o + s + 1], f + 6 * (o + s), f + 6 * (o + s + 1),
                             t0, dt, nots, trace, &err);
    }
    return err;
}

/* Per trajectory point: idx = round((ts-t0)/dt) clamped to [-2, nots+1] and
   flags bit0 = (ts <= tmin), bit1 = (ts < tmax) -- every quantity the deposit
   of src/particle.cpp:786-865 branches on (the clamp keeps all of them). */
void lwo_point_decisions(int64_t np, const double *t, const double *x, const double *obs,
                         double t0, double dt, int64_t nots, int64_t *idx, int32_t *flags)
{
    double tmin = t0 - dt * 0.5;
    double tmax = t0 + dt * ((double)nots - 0.5);
    for (int64_t i = 0; i < np; i++) {
        double ts = lwo_retarded_time(t[i], x + 3 * i, obs);
        double u = (ts - t0) / dt;
        if (u < -4.0) u = -4.0;
        if (u > (double)nots + 4.0) u = (double)nots + 4.0;
        int64_t k = (int64_t)round(u);
        if (k < -2) k = -2;
        if (k > nots + 1) k = nots + 1;
        idx[i] = k;
        flags[i] = (ts <= tmin ? 1 : 0) | (ts < tmax ? 2 : 0);
    }
}

/* The decisions of lwo_point_decisions for every (pixel, particle, point) of
   a screen, encoded as the device's decision record does
   (teufel_cuda_record_decisions): (idx + 4) | (flags << 27), at
   rec[(pixel * n_particles + m) * stride + i].  OpenMP over pixels. */
void lwo_screen_decisions(int64_t n_particles, const int64_t *offsets, const double *t,
                          const double *x, int64_t n_pix, const double *pix_pos,
                          const double *pix_t0, double dt, int64_t nots, int64_t stride,
                          int32_t *rec)
{
    int64_t p;
#pragma omp parallel for schedule(dynamic, 4)
    for (p = 0; p < n_pix; p++) {
        const double *obs = pix_pos + 3 * p;
        const double t0 = pix_t0[p];
        const double tmin = t0 - dt * 0.5;
        const double tmax = t0 + dt * ((double)nots - 0.5);
        for (int64_t m = 0; m < n_particles; m++) {
            int32_t *r = rec + (p * n_particles + m) * stride;
            for (int64_t i = offsets[m]; i < offsets[m + 1]; i++) {
                double ts = lwo_retarded_time(t[i], x + 3 * i, obs);
                double u = (ts - t0) / dt;
                if (u < -4.0) u = -4.0;
                if (u > (double)nots + 4.0) u = (double)nots + 4.0;
                int64_t k = (int64_t)round(u);
                if (k < -2) k = -2;
                if (k > nots + 1) k = nots + 1;
                int32_t fl = (ts <= tmin ? 1 : 0) | (ts < tmax ? 2 : 0);
                r[i - offsets[m]] = (int32_t)((k + 4) | ((int64_t)fl << 27));
            }
        }
    }
}

/* Per-point decision record used by the bin-index parity tests: for each
   step of particle m at observer obs, the pair (round((ts1-t0)/dt),
   round((ts2-t0)/dt)) and the case (0 = outside, 1 = starts before the
   window, 2 = inside).  Arrays have np-1 entries. */
void lwo_step_decisions(int64_t np, const double *t, const double *x, const double *obs,
                        double t0, double dt, int64_t nots, int64_t *idx1, int64_t *idx2,
                        int8_t *kase)
{
    double tmin = t0 - dt * 0.5;
    double tmax = t0 + dt * ((double)nots - 0.5);
    for (int64_t s = 0; s + 1 < np; s++) {
        double ts1 = lwo_retarded_time(t[s], x + 3 * s, obs);
        double ts2 = lwo_retarded_time(t[s + 1], x + 3 * (s + 1), obs);
        idx1[s] = (int64_t)round((ts1 - t0) / dt);
        idx2[s] = (int64_t)round((ts2 - t0) / dt);
        if (!((ts2 > tmin) && (ts1 < tmax))) kase[s] = 0;
        else if (ts1 <= tmin) kase[s] = 1;
        else kase[s] = 2;
    }
}

/* ---------------------------------------------------------------------------
 * The field at one observation time and place:
 *   ChargedParticle::RetardedField(double obs_time, Vector obs_pos)
 *                                               src/particle.cpp:612-769
 *   Bunch::RetardedField (sum in particle order)    src/bunch.cpp:729-737
 * -------------------------------------------------------------------------*/

/* The LW field of a source at SourceX moving with SourceBeta (gamma2 =
   gamma^2) and d(beta)/dt = betap, observed at o (src/particle.cpp:750-766). */
static void field_of_source(v3 o, v3 sx, v3 beta, v3 betap, double gamma2, double charge,
                            double *out6)
{
    v3 rv = v3_sub(o, sx);
    double R = v3_norm(rv);
    v3 n = rv;
    double nn = v3_norm(n);
    n.x /= nn; n.y /= nn; n.z /= nn;
    double scale = charge * LWO_E_CHARGE / (4.0 * LWO_PI * LWO_EPS0);
    double k3 = pow(1.0 - v3_dot(beta, n), 3.0);
    v3 E = v3_div(v3_sub(n, beta), R * R * k3 * gamma2);
    v3 acc = v3_cross(n, v3_cross(v3_sub(n, beta), betap));
    E = v3_add(E, v3_div(acc, R * k3 * LWO_C));
    E = v3_mul(E, scale);
    v3 B = v3_div(v3_cross(n, E), LWO_C);
    out6[0] = E.x; out6[1] = E.y; out6[2] = E.z;
    out6[3] = B.x; out6[4] = B.y; out6[5] = B.z;
}

/* One particle of np points (np >= 1).  Adds its field into acc6. */
static void retarded_field_particle(int64_t np, const double *T, const double *Xa,
                                    const double *Pa, const double *Aa, double charge,
                                    double obs_time, v3 o, double *acc6)
{
#define PT(a, i) ((v3){(a)[3 * (i)], (a)[3 * (i) + 1], (a)[3 * (i) + 2]})
    int64_t i1 = 0, i2 = np - 1;
    double R1 = v3_norm(v3_sub(o, PT(Xa, i1)));
    double t1 = obs_time - (T[i1] + R1 / LWO_C);
    double R2 = v3_norm(v3_sub(o, PT(Xa, i2)));
    double t2 = obs_time - (T[i2] + R2 / LWO_C);
    if (!(t2 <= 0.0)) return; /* no signal has arrived yet */
    v3 sx, beta, betap;
    double gamma2;
    if (t1 <= 0.0) {
        /* extrapolation to negative trajectory times (src/particle.cpp:639-659) */
        v3 Rc = v3_div(v3_sub(o, PT(Xa, 0)), LWO_C);
        beta = PT(Pa, 0);
        double bg2 = v3_abs2(beta);
        gamma2 = bg2 + 1.0;
        double gamma = sqrt(gamma2);
        beta = v3_div(beta, gamma);
        double t0 = obs_time;
        double bR = v3_dot(beta, Rc);
        double bb = v3_dot(beta, beta);
        double RR = v3_dot(Rc, Rc);
        double st = (t0 - bR - sqrt((t0 - bR) * (t0 - bR) - (1 - bb) * (t0 * t0 - RR))) / (1 - bb);
        sx = v3_add(PT(Xa, 0), v3_mul(v3_mul(beta, LWO_C), st));
        betap = (v3){0.0, 0.0, 0.0};
    } else {
        /* bisection to a single step (src/particle.cpp:666-685) */
        while (i2 - i1 > 1) {
            int64_t im = (i2 + i1) / 2;
            double Rm = v3_norm(v3_sub(o, PT(Xa, im)));
            double tm = obs_time - (T[im] + Rm / LWO_C);
            if (tm > 0.0) { i1 = im; t1 = tm; }
            else { i2 = im; t2 = tm; }
        }
        double frac = t1 / (t1 - t2);
        /* secant refinement (src/particle.cpp:693-733) */
        double tt1 = T[i1], tt2 = T[i2];
        v3 X1 = PT(Xa, i1), X2 = PT(Xa, i2);
        double st = tt1 * (1.0 - frac) + tt2 * frac;
        sx = v3_add(v3_mul(X1, 1.0 - frac), v3_mul(X2, frac));
        double R = v3_norm(v3_sub(o, sx));
        double dt = st + R / LWO_C - obs_time;
        double r1 = v3_norm(v3_sub(o, X1));
        double r2 = v3_norm(v3_sub(o, X2));
        double dtdfrac = (tt2 - tt1) + (r2 - r1) / LWO_C;
        double dfrac = dt / dtdfrac;
        int nref = 1;
        while (fabs(dfrac) > 1e-5 && nref < 10) {
            double last = dt;
            frac -= dfrac;
            st = tt1 * (1.0 - frac) + tt2 * frac;
            sx = v3_add(v3_mul(X1, 1.0 - frac), v3_mul(X2, frac));
            R = v3_norm(v3_sub(o, sx));
            dt = st + R / LWO_C - obs_time;
            dtdfrac = -(dt - last) / dfrac;
            dfrac = dt / dtdfrac;
            nref++;
        }
        frac -= dfrac;
        sx = v3_add(v3_mul(X1, 1.0 - frac), v3_mul(X2, frac));
        beta = v3_add(v3_mul(PT(Pa, i1), 1.0 - frac), v3_mul(PT(Pa, i2), frac));
        double bg2 = v3_abs2(beta);
        gamma2 = bg2 + 1.0;
        double gamma = sqrt(gamma2);
        beta = v3_div(beta, gamma);
        betap = v3_add(v3_mul(PT(Aa, i1), 1.0 - frac), v3_mul(PT(Aa, i2), frac));
        betap = v3_div(betap, gamma);
    }
    double f[6];
    field_of_source(o, sx, beta, betap, gamma2, charge, f);
    for (int k = 0; k < 6; k++) acc6[k] += f[k];
#undef PT
}

/* The summed field of all particles (charges in units of e) at obs_time on
   each of np observation points: out[np][6] is overwritten, as
   SnapshotObserver::integrate assigns (src/snapshot.cpp:72-80).  Returns
   LWO_ERR_RANGE if a particle has no trajectory point, where the reference
   throws RANGEexception (src/particle.cpp:615). */
int lwo_retarded_field_at(int64_t n_part, const int64_t *offsets, const double *charge,
                          const double *t, const double *x, const double *bg, const double *a,
                          double obs_time, int64_t np, const double *pos, double *out,
                          int nthreads)
{
    for (int64_t m = 0; m < n_part; m++)
        if (offsets[m + 1] - offsets[m] < 1) return LWO_ERR_RANGE;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
    for (int64_t p = 0; p < np; p++) {
        v3 o = {pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]};
        double acc[6] = {0, 0, 0, 0, 0, 0};
        for (int64_t m = 0; m < n_part; m++) {
            int64_t b = offsets[m];
            retarded_field_particle(offsets[m + 1] - b, t + b, x + 3 * b, bg + 3 * b, a + 3 * b,
                                    charge[m], obs_time, o, acc);
        }
        for (int k = 0; k < 6; k++) out[6 * p + k] = acc[k];
    }
    return LWO_OK;
}
