// ref_driver.cpp -- C entry points around the reference's own compiled code.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile together with the
// reference's unmodified src/{vector,fields,fieldtrace,particle,global}.cpp
// (compiled where they lie, into oracle/_ref/), and used only to produce the
// golden fixtures under tests/golden/ and to check the C restatement in
// oracle/lw_oracle.c.  Nothing on the product path loads it.
//
// What it exposes:
//  * ref_track: the reference's ChargedParticle::InitVay/StepVay
//    (src/particle.cpp:407-512) driven through a planar-undulator /
//    homogeneous field.  The undulator's LocalField (src/undulator.cpp:107-125)
//    is restated here because undulator.cpp needs muParser to compile.
//  * ref_integrate_screen: ChargedParticle::integrateFieldTrace
//    (src/particle.cpp:771-867) for every (pixel, particle), pixels in an
//    OpenMP loop as src/mesh.cpp:296 does, particles in bunch order
//    (src/bunch.cpp:739-745).  Particles are rebuilt from trajectory buffers
//    through the reference's public constructor
//    ChargedParticle(double *buffer, int nTraj, int nPre) (src/particle.cpp:121-158).
//  * ref_deposit_injected: the same integrateFieldTrace with injected arrival
//    times and fields, through a subclass that overrides the two virtual
//    retarded-point methods -- the mechanism the reference's own
//    known-answer test uses (tests/teufel.integrate_field.cpp:51-78).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include <omp.h>

#include "fields.h"
#include "fieldtrace.h"
#include "global.h"
#include "particle.h"
#include "vector.h"

namespace {

class HarnessField : public GeneralField {
public:
    bool has_und = false, has_hom = false;
    double b_peak = 0.0, lambda_u = 1.0, kz = 2.0 * Pi;
    int n_periods = 1;
    Vector origin = Vector(0.0, 0.0, 0.0);
    Vector hom_e = Vector(0.0, 0.0, 0.0), hom_b = Vector(0.0, 0.0, 0.0);

    bool is_external() override { return true; }

    ElMagField Field(double t, Vector X) override {
        ElMagField total = ElMagField();
        if (has_und) total += undulator(X - origin);
        if (has_hom) total += ElMagField(hom_e, hom_b);
        return total;
    }

private:
    ElMagField undulator(Vector X) {
        Vector E = Vector(0.0, 0.0, 0.0);
        Vector B = Vector(0.0, 0.0, 0.0);
        double z1 = -(n_periods + 1) * lambda_u / 2.0;
        double z2 = (n_periods + 1) * lambda_u / 2.0;
        if (z1 <= X.z && X.z < z2) {
            B.x = 0.0;
            B.y = b_peak * sin(kz * X.z) * cosh(kz * X.y);
            B.z = b_peak * cos(kz * X.z) * sinh(kz * X.y);
            if (X.z < z1 + lambda_u) B *= (X.z - z1) / lambda_u;
            if (z2 - lambda_u <= X.z) B *= (z2 - X.z) / lambda_u;
        }
        return ElMagField(E, B);
    }
};

class InjectedParticle : public ChargedParticle {
public:
    InjectedParticle(int np, const double* ts, const double* f) : ts_(ts), f_(f) { NP = np; }
    double RetardedTime(int index, Vector) override { return ts_[index]; }
    ElMagField RetardedField(int index, Vector) override {
        const double* v = f_ + 6 * index;
        return ElMagField(Vector(v[0], v[1], v[2]), Vector(v[3], v[4], v[5]));
    }

private:
    const double* ts_;
    const double* f_;
};

}  // namespace

extern "C" {

int ref_track(int64_t n_part, const double* init, double charge, double mass, const double* lat,
              double tstep, int64_t n_steps, double* out_t, double* out_x, double* out_p,
              double* out_a) {
    HarnessField fld;
    fld.has_und = lat[0] != 0.0;
    fld.b_peak = lat[1];
    fld.lambda_u = lat[2];
    fld.n_periods = (int)lat[3];
    fld.origin = Vector(lat[4], lat[5], lat[6]);
    fld.kz = 2.0 * Pi / fld.lambda_u;
    fld.has_hom = lat[7] != 0.0;
    fld.hom_e = Vector(lat[8], lat[9], lat[10]);
    fld.hom_b = Vector(lat[11], lat[12], lat[13]);
    const int64_t np = n_steps + 1;
    for (int64_t m = 0; m < n_part; m++) {
        const double* in = init + 7 * m;
        ChargedParticle p(charge, mass);
        p.initTrajectory(in[0], Vector(in[1], in[2], in[3]), Vector(in[4], in[5], in[6]),
                         Vector(0.0, 0.0, 0.0));
        p.InitVay(tstep, &fld);
        for (int64_t k = 0; k < n_steps; k++) p.StepVay(&fld);
        if (p.getNP() != np) return 2;
        for (int64_t k = 0; k < np; k++) {
            out_t[np * m + k] = p.TrajTime((int)k);
            Vector x = p.TrajPoint((int)k), q = p.TrajMomentum((int)k), a = p.TrajAccel((int)k);
            double* ox = out_x + 3 * (np * m + k);
            double* op = out_p + 3 * (np * m + k);
            double* oa = out_a + 3 * (np * m + k);
            ox[0] = x.x; ox[1] = x.y; ox[2] = x.z;
            op[0] = q.x; op[1] = q.y; op[2] = q.z;
            oa[0] = a.x; oa[1] = a.y; oa[2] = a.z;
        }
    }
    return 0;
}

// offsets[n_part+1] into the concatenated point arrays; charge in units of e
// (the reference's ChargedParticle::Charge); mass in electron masses.
int ref_integrate_screen(int64_t n_part, const int64_t* offsets, const double* charge,
                         const double* mass, const double* t, const double* x, const double* p,
                         const double* a, int64_t n_pix, const double* pix_pos,
                         const double* pix_t0, double dt, int64_t nots, double* out,
                         int nthreads) {
    std::vector<ChargedParticle*> parts;
    parts.reserve(n_part);
    for (int64_t m = 0; m < n_part; m++) {
        int64_t o = offsets[m], np = offsets[m + 1] - o;
        std::vector<double> buf(9 + 10 * np, 0.0);
        buf[0] = charge[m];
        buf[1] = mass[m];
        for (int64_t k = 0; k < np; k++) {
            double* b = buf.data() + 9 + 10 * k;
            b[0] = t[o + k];
            std::memcpy(b + 1, x + 3 * (o + k), 24);
            std::memcpy(b + 4, p + 3 * (o + k), 24);
            std::memcpy(b + 7, a + 3 * (o + k), 24);
        }
        parts.push_back(new ChargedParticle(buf.data(), (int)np, 0));
    }
    int err = 0;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
    for (int64_t ip = 0; ip < n_pix; ip++) {
        FieldTrace tr(pix_t0[ip], dt, (std::size_t)nots);
        double* o = out + 6 * nots * ip;
        tr.set_buffer((ElMagField*)o, (std::size_t)nots);
        const double* pp = pix_pos + 3 * ip;
        try {
            for (int64_t m = 0; m < n_part; m++)
                parts[m]->integrateFieldTrace(Vector(pp[0], pp[1], pp[2]), &tr);
        } catch (...) {
#pragma omp critical
            err = 4;
        }
        tr.get_buffer((ElMagField*)o, (std::size_t)nots);
    }
    for (auto* q : parts) delete q;
    return err;
}

// The reference's ChargedParticle::RetardedField(double, Vector) summed over
// the particles in order as Bunch::RetardedField does (src/bunch.cpp:729-737),
// on np observation points at obs_time; out[np][6] is overwritten.
int ref_retarded_field_at(int64_t n_part, const int64_t* offsets, const double* charge,
                          const double* mass, const double* t, const double* x, const double* p,
                          const double* a, double obs_time, int64_t n_obs, const double* pos,
                          double* out) {
    std::vector<ChargedParticle*> parts;
    parts.reserve(n_part);
    for (int64_t m = 0; m < n_part; m++) {
        int64_t o = offsets[m], np = offsets[m + 1] - o;
        std::vector<double> buf(9 + 10 * np, 0.0);
        buf[0] = charge[m];
        buf[1] = mass[m];
        for (int64_t k = 0; k < np; k++) {
            double* b = buf.data() + 9 + 10 * k;
            b[0] = t[o + k];
            std::memcpy(b + 1, x + 3 * (o + k), 24);
            std::memcpy(b + 4, p + 3 * (o + k), 24);
            std::memcpy(b + 7, a + 3 * (o + k), 24);
        }
        parts.push_back(new ChargedParticle(buf.data(), (int)np, 0));
    }
    int err = 0;
    for (int64_t ip = 0; ip < n_obs && !err; ip++) {
        const double* pp = pos + 3 * ip;
        ElMagField f;
        try {
            for (int64_t m = 0; m < n_part; m++)
                f += parts[m]->RetardedField(obs_time, Vector(pp[0], pp[1], pp[2]));
        } catch (...) {
            err = 4;
        }
        Vector E = f.E(), B = f.B();
        double* o = out + 6 * ip;
        o[0] = E.x; o[1] = E.y; o[2] = E.z;
        o[3] = B.x; o[4] = B.y; o[5] = B.z;
    }
    for (auto* q : parts) delete q;
    return err;
}

int ref_deposit_injected(int64_t n_part, const int64_t* offsets, const double* ts,
                         const double* f, double t0, double dt, int64_t nots, double* trace) {
    FieldTrace tr(t0, dt, (std::size_t)nots);
    tr.set_buffer((ElMagField*)trace, (std::size_t)nots);
    int err = 0;
    try {
        for (int64_t m = 0; m < n_part; m++) {
            int64_t o = offsets[m];
            InjectedParticle q((int)(offsets[m + 1] - o), ts + o, f + 6 * o);
            q.integrateFieldTrace(Vector(0.0, 0.0, 0.0), &tr);
        }
    } catch (...) {
        err = 4;
    }
    tr.get_buffer((ElMagField*)trace, (std::size_t)nots);
    return err;
}

}  // extern "C"

// The reference's ChargedParticle::CoordinatesAtTime (src/particle.cpp:514-558)
// of every particle at one time: out[n_part][6] = position, beta*gamma.
extern "C" int ref_coordinates_at_time(int64_t n_part, const int64_t* offsets, const double* t,
                                       const double* x, const double* p, double time,
                                       double* out) {
    for (int64_t m = 0; m < n_part; m++) {
        int64_t o = offsets[m], np = offsets[m + 1] - o;
        std::vector<double> buf(9 + 10 * np, 0.0);
        buf[0] = -1.0;
        buf[1] = 1.0;
        for (int64_t k = 0; k < np; k++) {
            double* b = buf.data() + 9 + 10 * k;
            b[0] = t[o + k];
            std::memcpy(b + 1, x + 3 * (o + k), 24);
            std::memcpy(b + 4, p + 3 * (o + k), 24);
        }
        ChargedParticle part(buf.data(), (int)np, 0);
        Vector X, BG;
        part.CoordinatesAtTime(time, &X, &BG);
        double* q = out + 6 * m;
        q[0] = X.x; q[1] = X.y; q[2] = X.z;
        q[3] = BG.x; q[4] = BG.y; q[5] = BG.z;
    }
    return 0;
}
