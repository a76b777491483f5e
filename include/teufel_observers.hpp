// teufel_observers.hpp -- C++ host layer over the C-ABI (teufel_cuda.h) with
// the interface of TEUFEL's observers, for code written against them.
//
// Mirrors, with the same member names, argument meaning and error behaviour:
//   BaseObserver / Observer<SourceT>     src/observer.h:43-146
//   ScreenObserver<Beam>                 src/screen.h, src/screen.cpp:34-146, 240-560
//   MeshedScreen<Beam> (read, init, integrate, buffer, writeFile, totalEnergy)
//                                        src/mesh.cpp:31-278, 289-316, 376-754
// HDF5 files are read and written by teufel_hdf5_read.hpp / teufel_hdf5_write.hpp
// (no HDF5 library needed); the PointObserver trace is written as SDDS.
//   PointObserver<Beam>                  src/point_observer.cpp:30-110
//   FieldTrace (t0, dt, N, add, buffer)  src/fieldtrace.h, src/fieldtrace.cpp
//   IOexception                          src/global.h:75-84
// integrate() runs on the GPU through teufel_cuda_integrate_screen /
// teufel_cuda_integrate_point; there is no CPU path.  A non-zero status is
// rethrown as IOexception carrying the C-ABI's message, as the reference
// throws IOexception from FieldTrace::add for out-of-range deposits.
//
// The field source (the reference's Beam/Bunch) is a TrajectorySource: the
// particles' trajectory arrays, uploaded once on first use and kept on the
// device for every observer that integrates from it.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "teufel_cuda.h"
#include "teufel_hdf5_read.hpp"
#include "teufel_hdf5_write.hpp"

namespace teufel_gb300 {

class IOexception : public std::exception {
public:
    explicit IOexception(std::string m) : msg(std::move(m)) {}
    const char* what() const throw() override { return msg.c_str(); }

private:
    std::string msg;
};

inline void check_status(int st, const char* where) {
    if (st != TEUFEL_OK)
        throw IOexception(std::string(where) + " - " + teufel_cuda_status_string(st));
}

struct Vector {
    double x = 0.0, y = 0.0, z = 0.0;
    Vector() = default;
    Vector(double a, double b, double c) : x(a), y(b), z(c) {}
    Vector operator+(const Vector& o) const { return Vector(x + o.x, y + o.y, z + o.z); }
    Vector operator*(double f) const { return Vector(x * f, y * f, z * f); }
    Vector operator-(const Vector& o) const { return Vector(x - o.x, y - o.y, z - o.z); }
    Vector& operator+=(const Vector& o) {
        x += o.x;
        y += o.y;
        z += o.z;
        return *this;
    }
    double norm() const { return std::sqrt(x * x + y * y + z * z); }
    // divides by the norm unguarded, as src/vector.cpp:137-143 does
    void normalize() {
        const double n = norm();
        x /= n;
        y /= n;
        z /= n;
    }
};

inline double dot(const Vector& a, const Vector& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vector cross(const Vector& a, const Vector& b) {
    return Vector(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// vacuum permeability [Vs/Am], as the reference defines it (src/global.h:43)
constexpr double kMuNull = 4.0 * 3.1415926535897932384626433832795029 * 1e-7;

// One electromagnetic sample: Ex, Ey, Ez, Bx, By, Bz (the ElMagField layout).
struct ElMagField {
    double c[6] = {0, 0, 0, 0, 0, 0};
    Vector E() const { return Vector(c[0], c[1], c[2]); }
    Vector B() const { return Vector(c[3], c[4], c[5]); }
};

// Trajectories of a particle set (what Beam/Bunch hold as ChargedParticle
// Time/X/P/A arrays, src/particle.h:417-427).
class TrajectorySource {
public:
    TrajectorySource() = default;
    TrajectorySource(const TrajectorySource&) = delete;
    TrajectorySource& operator=(const TrajectorySource&) = delete;
    ~TrajectorySource() { release(); }

    // Append one particle: charge [C] (ChargedParticle::getCharge()),
    // n trajectory points of time [s], position [m], beta*gamma and
    // d(beta*gamma)/dt [1/s] (TrajTime/TrajPoint/TrajMomentum/TrajAccel).
    void Add(double charge_C, int n, const double* t, const double* x, const double* bg,
             const double* a) {
        release();
        charge.push_back(charge_C);
        npts.push_back(n);
        T.insert(T.end(), t, t + n);
        X.insert(X.end(), x, x + 3 * (size_t)n);
        P.insert(P.end(), bg, bg + 3 * (size_t)n);
        A.insert(A.end(), a, a + 3 * (size_t)n);
    }
    int getNOP() const { return (int)npts.size(); }

    // Position and beta*gamma of particle i at a time, interpolated linearly
    // between the bracketing trajectory points; zero outside the trajectory
    // (ChargedParticle::CoordinatesAtTime, src/particle.cpp:514-558).
    void CoordinatesAtTime(int i, double time, Vector* position, Vector* momentum) const {
        std::size_t first = 0;
        for (int k = 0; k < i; k++) first += (std::size_t)npts[k];
        const int np = npts[i];
        *position = Vector(0.0, 0.0, 0.0);
        *momentum = Vector(0.0, 0.0, 0.0);
        if (np < 1) return;
        int i1 = 0, i2 = np - 1;
        double t1 = T[first], t2 = T[first + i2];
        if (!(time >= t1 && time <= t2)) return;
        while (i2 - i1 > 1) {
            const int im = (i2 + i1) / 2;
            const double t = T[first + im];
            if (t < time) {
                i1 = im;
                t1 = t;
            } else {
                i2 = im;
                t2 = t;
            }
        }
        const double* x1 = &X[3 * (first + i1)];
        const double* p1 = &P[3 * (first + i1)];
        if (i2 == i1) {
            *position = Vector(x1[0], x1[1], x1[2]);
            *momentum = Vector(p1[0], p1[1], p1[2]);
            return;
        }
        const double* x2 = &X[3 * (first + i2)];
        const double* p2 = &P[3 * (first + i2)];
        const double frac = (time - t1) / (t2 - t1);
        *position = Vector(x1[0], x1[1], x1[2]) * (1.0 - frac) + Vector(x2[0], x2[1], x2[2]) * frac;
        *momentum = Vector(p1[0], p1[1], p1[2]) * (1.0 - frac) + Vector(p2[0], p2[1], p2[2]) * frac;
    }

    // the device-resident set, uploaded on first use
    const teufel_traj_set* device() {
        if (!handle)
            check_status(teufel_cuda_traj_upload((int)npts.size(), npts.data(), charge.data(),
                                                 T.data(), X.data(), P.data(), A.data(), &handle),
                         "TrajectorySource::device");
        return handle;
    }
    void release() {
        if (handle) teufel_cuda_traj_free(handle);
        handle = nullptr;
    }

private:
    std::vector<double> charge, T, X, P, A;
    std::vector<int> npts;
    teufel_traj_set* handle = nullptr;
};

// FieldTrace: N samples of width dt centred on t0 + i*dt (src/fieldtrace.h).
class FieldTrace {
public:
    FieldTrace(double t0_p, double dt_p, std::size_t N_p) : t0(t0_p), dt(dt_p), N(N_p), f(N_p) {}
    double get_t0() const { return t0; }
    double get_dt() const { return dt; }
    std::size_t get_N() const { return N; }
    double get_time(std::size_t i) const {
        if (i >= N) throw IOexception("FieldTrace::get_time - index out of range.");
        return t0 + i * dt;
    }
    ElMagField get_field(std::size_t i) const {
        if (i >= N) throw IOexception("FieldTrace::get_field - index out of range.");
        return f[i];
    }
    void zero() { std::fill(f.begin(), f.end(), ElMagField()); }
    double* data() { return f.empty() ? nullptr : f[0].c; }

private:
    double t0, dt;
    std::size_t N;
    std::vector<ElMagField> f;
};

class BaseObserver {
public:
    virtual ~BaseObserver() {}
    virtual void integrate() = 0;
    virtual std::size_t getBufferSize() = 0;
    virtual double* getBuffer() = 0;  // new[]-allocated, freed by the caller
    virtual void fromBuffer(double* buffer, std::size_t size) = 0;
    virtual void generateOutput() = 0;
};

template <typename SourceT>
class Observer : public BaseObserver {
public:
    virtual void setSource(SourceT* src) { source = src; }
    SourceT* source = nullptr;
};

// Nx x Ny rectangular screen (src/screen.cpp:34-110).
class ScreenObserver : public Observer<TrajectorySource> {
public:
    // filename is where generateOutput() writes the HDF5 file
    ScreenObserver(std::string filename, Vector position, Vector dx, Vector dy, unsigned int nx,
                   unsigned int ny, double t0, double dt, double dtx, double dty, unsigned int nots)
        : FileName(std::move(filename)), Origin(position), dX(dx), dY(dy), Nx(nx), Ny(ny),
          t0_obs(t0), dt_obs(dt), dtx_obs(dtx), dty_obs(dty), NOTS(nots),
          buf((std::size_t)nx * ny * nots * 6, 0.0) {
        normal = cross(dX, dY) * -1.0;  // the backward normal, src/screen.cpp:52-53
        normal.normalize();
    }
    ScreenObserver(Vector position, Vector dx, Vector dy, unsigned int nx, unsigned int ny,
                   double t0, double dt, double dtx, double dty, unsigned int nots)
        : ScreenObserver(std::string(), position, dx, dy, nx, ny, t0, dt, dtx, dty, nots) {}
    Vector getNormal() const { return normal; }

    // center index is Nx/2, Ny/2 with integer division (src/screen.cpp:97-103)
    Vector CellPosition(unsigned int ix, unsigned int iy) const {
        return Origin + dX * (double)((int)ix - (int)Nx / 2) + dY * (double)((int)iy - (int)Ny / 2);
    }
    double CellTimeZero(unsigned int ix, unsigned int iy) const {
        return t0_obs + dtx_obs * (double)((int)ix - (int)Nx / 2) +
               dty_obs * (double)((int)iy - (int)Ny / 2);
    }

    void integrate() override {
        if (!source) throw IOexception("ScreenObserver::integrate - no source set");
        const std::size_t np = (std::size_t)Nx * Ny;
        std::vector<double> pos(3 * np), t0(np);
        for (unsigned int ix = 0; ix < Nx; ix++)
            for (unsigned int iy = 0; iy < Ny; iy++) {
                const std::size_t p = (std::size_t)ix * Ny + iy;
                Vector c = CellPosition(ix, iy);
                pos[3 * p] = c.x;
                pos[3 * p + 1] = c.y;
                pos[3 * p + 2] = c.z;
                t0[p] = CellTimeZero(ix, iy);
            }
        // traces still cleared (constructed or zero()ed): stored, not added,
        // so that the call does not upload them
        teufel_options opt;
        teufel_cuda_default_options(&opt);
        opt.overwrite_out = cleared ? 1 : 0;
        cleared = false;
        check_status(teufel_cuda_integrate_screen_ex(source->device(), pos.data(), t0.data(),
                                                     dt_obs, (int)NOTS, (int)np, buf.data(), &opt,
                                                     nullptr),
                     "ScreenObserver::integrate");
    }

    ElMagField getField(unsigned int ix, unsigned int iy, unsigned int it) const {
        if (ix >= Nx || iy >= Ny || it >= NOTS)
            throw IOexception("ScreenObserver::getField() - requested index out of range.");
        ElMagField f;
        std::memcpy(f.c, &buf[(((std::size_t)ix * Ny + iy) * NOTS + it) * 6], sizeof f.c);
        return f;
    }
    std::size_t getBufferSize() override { return (std::size_t)Nx * Ny * NOTS * 6; }
    double* getBuffer() override {
        double* b = new double[getBufferSize()];
        std::memcpy(b, buf.data(), sizeof(double) * getBufferSize());
        return b;
    }
    void fromBuffer(double* buffer, std::size_t size) override {
        if (size != getBufferSize())
            throw IOexception("ScreenObserver::fromBuffer() - buffer size mismatch.");
        std::memcpy(buf.data(), buffer, sizeof(double) * size);
        cleared = false;
    }
    // The HDF5 layout of src/screen.cpp:298-560: ObservationPosition
    // [Nx][Ny][3] (attributes Nx, Ny), Screen [4][3] = origin, normal, dX, dY
    // (Nx, Ny, NOTS, t0, dt, dtx, dty) and ElMagField [Nx][Ny][NOTS][6]
    // (t0, dt, NOTS).
    void WriteTimeDomainFieldHDF5() {
        if (FileName.empty())
            throw IOexception("ScreenObserver::WriteTimeDomainFieldHDF5 - no file name given");
        std::vector<double> pos((std::size_t)Nx * Ny * 3);
        for (unsigned int ix = 0; ix < Nx; ix++)
            for (unsigned int iy = 0; iy < Ny; iy++) {
                const Vector c = CellPosition(ix, iy);
                double* q = &pos[((std::size_t)ix * Ny + iy) * 3];
                q[0] = c.x;
                q[1] = c.y;
                q[2] = c.z;
            }
        const double screen[12] = {Origin.x, Origin.y, Origin.z, normal.x, normal.y, normal.z,
                                   dX.x,     dX.y,     dX.z,     dY.x,     dY.y,     dY.z};
        using h5::AttrOut;
        try {
            h5::Writer w;
            w.add("ObservationPosition", {Nx, Ny, 3}, pos.data(),
                  {AttrOut::Int("Nx", (int32_t)Nx), AttrOut::Int("Ny", (int32_t)Ny)});
            w.add("Screen", {4, 3}, screen,
                  {AttrOut::Int("Nx", (int32_t)Nx), AttrOut::Int("Ny", (int32_t)Ny),
                   AttrOut::Int("NOTS", (int32_t)NOTS), AttrOut::Double("t0", t0_obs),
                   AttrOut::Double("dt", dt_obs), AttrOut::Double("dtx", dtx_obs),
                   AttrOut::Double("dty", dty_obs)});
            w.add("ElMagField", {Nx, Ny, NOTS, 6}, buf.data(),
                  {AttrOut::Double("t0", t0_obs), AttrOut::Double("dt", dt_obs),
                   AttrOut::Int("NOTS", (int32_t)NOTS)});
            w.write(FileName);
        } catch (const h5::Error& e) {
            throw IOexception(std::string("ScreenObserver::WriteTimeDomainFieldHDF5 - ") + e.what());
        }
    }
    void generateOutput() override { WriteTimeDomainFieldHDF5(); }
    void zero() {
        std::fill(buf.begin(), buf.end(), 0.0);
        cleared = true;
    }

private:
    std::string FileName;
    Vector Origin, dX, dY, normal;
    unsigned int Nx, Ny;
    double t0_obs, dt_obs, dtx_obs, dty_obs;
    unsigned int NOTS;
    std::vector<double> buf;  // [Nx][Ny][NOTS][6]
    bool cleared = true;      // buf holds only zeros
};

// A screen of triangular cells, each observed at one point with its own trace
// start time (src/mesh.h, src/mesh.cpp).
class MeshedScreen : public Observer<TrajectorySource> {
public:
    // Reads the mesh as MeshedScreen(std::string) does (src/mesh.cpp:31-218):
    // MeshCornerPoints [Ncp][3] (attribute Ncp), ObservationPosition [Np][3]
    // (attribute Np), MeshTriangles [Np][3] corner indices, and when present
    // ObservationTime [Np] (attributes Nt, dt) and ElMagField [Np][Nt][6].
    // Without ObservationTime the traces are empty (t0 = dt = 0, Nt = 0).
    explicit MeshedScreen(const std::string& filename) : FileName(filename) {
        try {
            load(filename);
        } catch (const h5::Error& e) {
            throw IOexception(std::string("MeshedScreen - ") + e.what());
        }
    }
    // A mesh given directly: observation points with their start times.
    MeshedScreen(std::vector<Vector> points, std::vector<double> t0, double dt, int nt)
        : pts(std::move(points)), T0(std::move(t0)), dt_obs(dt), Nt(nt),
          buf(pts.size() * (std::size_t)nt * 6, 0.0) {
        if (T0.size() != pts.size()) throw IOexception("MeshedScreen - t0 size mismatch.");
    }
    // A triangle mesh given directly: corner points, the cells' corner
    // indices [Np][3], and per cell the observation point and start time.
    MeshedScreen(std::string filename, std::vector<Vector> corners, std::vector<int> triangles,
                 std::vector<Vector> points, std::vector<double> t0, double dt, int nt)
        : MeshedScreen(std::move(points), std::move(t0), dt, nt) {
        FileName = std::move(filename);
        corner = std::move(corners);
        if (triangles.size() != 3 * pts.size())
            throw IOexception("MeshedScreen - triangle count mismatch.");
        tri.assign(triangles.begin(), triangles.end());
        for (int64_t c : tri)
            if (c < 0 || c >= (int64_t)corner.size())
                throw IOexception("MeshedScreen - MeshTriangles index out of range");
    }
    int get_Np() const { return (int)pts.size(); }
    int get_Nt() const { return Nt; }
    double get_dt() const { return dt_obs; }
    Vector get_point(int ip) const { return pts[ip]; }
    double get_t0(int ip) const { return T0[ip]; }
    Vector get_xi(int ip) const { return xi[ip]; }
    Vector get_eta(int ip) const { return eta[ip]; }
    Vector get_normal(int ip) const { return normal[ip]; }
    double get_area(int ip) const { return area[ip]; }
    double getTotalArea() const { return total_area; }

    // Cell areas, unit normals and the cell-local (xi, eta, normal) frames,
    // as src/mesh.cpp:227-278 computes them.
    void init() {
        if (tri.size() != 3 * pts.size())
            throw IOexception("MeshedScreen::init - the screen has no triangle mesh.");
        const std::size_t np = pts.size();
        area.assign(np, 0.0);
        normal.assign(np, Vector());
        xi.assign(np, Vector());
        eta.assign(np, Vector());
        total_area = 0.0;
        Vector avg;
        for (std::size_t ip = 0; ip < np; ip++) {
            const Vector& p1 = corner[(std::size_t)tri[3 * ip]];
            const Vector& p2 = corner[(std::size_t)tri[3 * ip + 1]];
            const Vector& p3 = corner[(std::size_t)tri[3 * ip + 2]];
            Vector n = cross(p3 - p1, p2 - p1);
            area[ip] = n.norm() * 0.5;
            total_area += area[ip];
            n.normalize();
            normal[ip] = n;
            avg += n;
        }
        avg.normalize();
        for (std::size_t ip = 0; ip < np; ip++) {
            if (avg.y < 0.7) {  // xi in the x-z plane
                xi[ip] = cross(Vector(0.0, 1.0, 0.0), normal[ip]);
                xi[ip].normalize();
                eta[ip] = cross(normal[ip], xi[ip]);
                eta[ip].normalize();
            } else {  // eta in the y-z plane
                eta[ip] = cross(normal[ip], Vector(1.0, 0.0, 0.0));
                eta[ip].normalize();
                xi[ip] = cross(eta[ip], normal[ip]);
                xi[ip].normalize();
            }
        }
    }

    ElMagField getField(int ip, int it) const {
        if (ip < 0 || ip >= (int)pts.size() || it < 0 || it >= Nt)
            throw IOexception("MeshedScreen::getField() - index out of range.");
        ElMagField f;
        std::memcpy(f.c, &buf[((std::size_t)ip * Nt + it) * 6], sizeof f.c);
        return f;
    }

    // dt * sum over the trace of E x B / mu0 (FieldTrace::Poynting,
    // src/fieldtrace.cpp:192-198)
    Vector Poynting(int ip) const {
        Vector sum;
        for (int it = 0; it < Nt; it++) {
            const double* f = &buf[((std::size_t)ip * Nt + it) * 6];
            sum += cross(Vector(f[0], f[1], f[2]), Vector(f[3], f[4], f[5])) * (1.0 / kMuNull);
        }
        return sum * dt_obs;
    }

    // Energy through the screen [J], flow against the normal counted
    // positive (src/mesh.cpp:744-754).  init() must have run.
    double totalEnergy() const {
        if (area.size() != pts.size())
            throw IOexception("MeshedScreen::totalEnergy - init() has not been called.");
        double total = 0.0;
        for (int ip = 0; ip < (int)pts.size(); ip++) total -= area[ip] * dot(Poynting(ip), normal[ip]);
        return total;
    }

    void integrate() override {
        if (!source) throw IOexception("MeshedScreen::integrate - no source set");
        if (Nt == 0 || pts.empty()) return;
        std::vector<double> pos(3 * pts.size());
        for (std::size_t i = 0; i < pts.size(); i++) {
            pos[3 * i] = pts[i].x;
            pos[3 * i + 1] = pts[i].y;
            pos[3 * i + 2] = pts[i].z;
        }
        teufel_options opt;
        teufel_cuda_default_options(&opt);
        opt.overwrite_out = cleared ? 1 : 0;
        cleared = false;
        check_status(teufel_cuda_integrate_screen_ex(source->device(), pos.data(), T0.data(),
                                                     dt_obs, Nt, (int)pts.size(), buf.data(), &opt,
                                                     nullptr),
                     "MeshedScreen::integrate");
    }
    std::size_t getBufferSize() override { return pts.size() * (std::size_t)Nt * 6; }
    double* getBuffer() override {
        double* b = new double[getBufferSize()];
        std::memcpy(b, buf.data(), sizeof(double) * getBufferSize());
        return b;
    }
    void fromBuffer(double* buffer, std::size_t size) override {
        if (size != getBufferSize())
            throw IOexception("MeshedScreen::fromBuffer() - buffer size mismatch.");
        std::memcpy(buf.data(), buffer, sizeof(double) * size);
        cleared = false;
    }
    // The HDF5 layout of src/mesh.cpp:428-736, which the file constructor
    // reads back: MeshCornerPoints [Ncp][3] (Ncp), ObservationPosition
    // [Np][3] (Np), MeshTriangles [Np][3] (Ntri), ObservationTime [Np]
    // (Nt, dt) and ElMagField [Np][Nt][6].
    void writeFile(const std::string& filename) {
        if (tri.size() != 3 * pts.size())
            throw IOexception("MeshedScreen::writeFile - the screen has no triangle mesh.");
        const uint64_t ncp = corner.size(), np = pts.size();
        std::vector<double> cp(3 * ncp), pp(3 * np);
        for (std::size_t i = 0; i < ncp; i++) {
            cp[3 * i] = corner[i].x;
            cp[3 * i + 1] = corner[i].y;
            cp[3 * i + 2] = corner[i].z;
        }
        for (std::size_t i = 0; i < np; i++) {
            pp[3 * i] = pts[i].x;
            pp[3 * i + 1] = pts[i].y;
            pp[3 * i + 2] = pts[i].z;
        }
        std::vector<int32_t> tr(tri.begin(), tri.end());
        using h5::AttrOut;
        try {
            h5::Writer w;
            w.add("MeshCornerPoints", {ncp, 3}, cp.data(), {AttrOut::Int("Ncp", (int32_t)ncp)});
            w.add("ObservationPosition", {np, 3}, pp.data(), {AttrOut::Int("Np", (int32_t)np)});
            w.add("MeshTriangles", {np, 3}, tr.data(), {AttrOut::Int("Ntri", (int32_t)np)});
            w.add("ObservationTime", {np}, T0.data(),
                  {AttrOut::Int("Nt", Nt), AttrOut::Double("dt", dt_obs)});
            w.add("ElMagField", {np, (uint64_t)Nt, 6}, buf.data());
            w.write(filename);
        } catch (const h5::Error& e) {
            throw IOexception(std::string("MeshedScreen::writeFile - ") + e.what());
        }
    }
    void writeFile() { writeFile(FileName); }
    void generateOutput() override { writeFile(); }
    void zero() {
        std::fill(buf.begin(), buf.end(), 0.0);
        cleared = true;
    }

private:
    void load(const std::string& filename) {
        h5::File f(filename);
        h5::Dataset d = f.dataset("MeshCornerPoints");
        const int64_t ncp = h5::File::attr_int(d, "Ncp");
        std::vector<double> v = f.read_double(d);
        if (ncp < 0 || v.size() != 3 * (std::size_t)ncp)
            throw IOexception("MeshedScreen - error reading dataset MeshCornerPoints");
        corner.resize((std::size_t)ncp);
        for (std::size_t i = 0; i < corner.size(); i++) corner[i] = Vector(v[3 * i], v[3 * i + 1], v[3 * i + 2]);

        d = f.dataset("ObservationPosition");
        const int64_t np = h5::File::attr_int(d, "Np");
        v = f.read_double(d);
        if (np < 0 || v.size() != 3 * (std::size_t)np)
            throw IOexception("MeshedScreen - error reading dataset ObservationPosition");
        pts.resize((std::size_t)np);
        for (std::size_t i = 0; i < pts.size(); i++) pts[i] = Vector(v[3 * i], v[3 * i + 1], v[3 * i + 2]);

        tri = f.read_int(f.dataset("MeshTriangles"));
        if (tri.size() != 3 * pts.size())
            throw IOexception("MeshedScreen - error reading dataset MeshTriangles");
        for (int64_t c : tri)
            if (c < 0 || c >= ncp) throw IOexception("MeshedScreen - MeshTriangles index out of range");

        if (f.exists("ObservationTime")) {
            d = f.dataset("ObservationTime");
            const int64_t nt = h5::File::attr_int(d, "Nt");
            if (nt < 0 || nt > (int64_t)1 << 30)
                throw IOexception("MeshedScreen - error reading dataset ObservationTime attribute Nt");
            Nt = (int)nt;
            dt_obs = h5::File::attr_double(d, "dt");
            T0 = f.read_double(d);
            if (T0.size() != pts.size())
                throw IOexception("MeshedScreen - error reading dataset ObservationTime");
        } else {
            Nt = 0;
            dt_obs = 0.0;
            T0.assign(pts.size(), 0.0);
        }
        buf.assign(pts.size() * (std::size_t)Nt * 6, 0.0);
        if (f.exists("ElMagField")) {
            v = f.read_double(f.dataset("ElMagField"));
            if (v.size() != buf.size()) throw IOexception("MeshedScreen - error reading dataset ElMagField");
            buf = std::move(v);
            cleared = false;
        }
    }

    std::string FileName;
    std::vector<Vector> corner;   // MeshCornerPoints
    std::vector<int64_t> tri;     // [Np][3] corner indices
    std::vector<Vector> pts;
    std::vector<double> T0;
    double dt_obs = 0.0;
    int Nt = 0;
    std::vector<double> buf;  // [Np][Nt][6]
    bool cleared = true;      // buf holds only zeros
    std::vector<Vector> xi, eta, normal;
    std::vector<double> area;
    double total_area = 0.0;
};

// The trace of one observation point as an SDDS (version 1) file in ASCII
// mode, with the layout PointObserver::WriteTimeDomainFieldSDDS writes
// (src/point_observer.cpp:120-181): parameters NumberTimeSteps (long), t0 and
// dt (double); columns t [s], Ex, Ey, Ez [V/m] and Bx, By, Bz [T] (double);
// one page of N rows.  Written from the SDDS format description; values carry
// 17 significant digits, so they read back exactly.
inline void write_trace_sdds(const std::string& filename, double t0, double dt, std::size_t N,
                             const double* f) {
    std::FILE* fp = std::fopen(filename.c_str(), "w");
    if (!fp)
        throw IOexception("PointObserver::WriteTimeDomainFieldSDDS - error in InitializeOutput()");
    std::fprintf(fp, "SDDS1\n");
    std::fprintf(fp, "&parameter name=NumberTimeSteps, type=long, &end\n");
    std::fprintf(fp, "&parameter name=t0, type=double, &end\n");
    std::fprintf(fp, "&parameter name=dt, type=double, &end\n");
    const char* cols[7][3] = {{"t", "s", "time"},
                              {"Ex", "V/m", "\"electric field\""},
                              {"Ey", "V/m", "\"electric field\""},
                              {"Ez", "V/m", "\"electric field\""},
                              {"Bx", "T", "\"magnetic field\""},
                              {"By", "T", "\"magnetic field\""},
                              {"Bz", "T", "\"magnetic field\""}};
    for (auto& c : cols)
        std::fprintf(fp, "&column name=%s, symbol=%s, units=%s, description=%s, type=double, &end\n",
                     c[0], c[0], c[1], c[2]);
    std::fprintf(fp, "&data mode=ascii, &end\n");
    std::fprintf(fp, "! page number 1\n");
    std::fprintf(fp, "%zu\n%.17g\n%.17g\n", N, t0, dt);
    std::fprintf(fp, "%zu\n", N);
    for (std::size_t i = 0; i < N; i++) {
        std::fprintf(fp, "%.17g", t0 + (double)i * dt);
        for (int c = 0; c < 6; c++) std::fprintf(fp, " %.17g", f[6 * i + c]);
        std::fprintf(fp, "\n");
    }
    if (std::fclose(fp) != 0)
        throw IOexception("PointObserver::WriteTimeDomainFieldSDDS - error in Terminate()");
}

// One observation point (src/point_observer.cpp:30-110, 120-186).
class PointObserver : public Observer<TrajectorySource> {
public:
    PointObserver(std::string filename, Vector position, double t0, double dt, std::size_t nots)
        : FileName(std::move(filename)), Pos(position), trace(t0, dt, nots) {}
    PointObserver(Vector position, double t0, double dt, std::size_t nots)
        : Pos(position), trace(t0, dt, nots) {}
    void WriteTimeDomainFieldSDDS() {
        // B in Tesla: the C-ABI delivers the reference's getBuffer() layout
        write_trace_sdds(FileName, trace.get_t0(), trace.get_dt(), trace.get_N(), trace.data());
    }
    void generateOutput() override { WriteTimeDomainFieldSDDS(); }
    void integrate() override {
        if (!source) throw IOexception("PointObserver::integrate - no source set");
        const double p[3] = {Pos.x, Pos.y, Pos.z};
        check_status(teufel_cuda_integrate_point(source->device(), p, trace.get_t0(),
                                                 trace.get_dt(), (int)trace.get_N(), trace.data(),
                                                 nullptr),
                     "PointObserver::integrate");
    }
    ElMagField getField(std::size_t it) const { return trace.get_field(it); }
    std::size_t getBufferSize() override { return 6 * trace.get_N(); }
    double* getBuffer() override {
        double* b = new double[getBufferSize()];
        if (getBufferSize()) std::memcpy(b, trace.data(), sizeof(double) * getBufferSize());
        return b;
    }
    void fromBuffer(double* buffer, std::size_t size) override {
        if (size != getBufferSize())
            throw IOexception("PointObserver::fromBuffer() - buffer size mismatch.");
        if (size) std::memcpy(trace.data(), buffer, sizeof(double) * size);
    }

private:
    std::string FileName;
    Vector Pos;
    FieldTrace trace;
};

// The field of the source on an Nx x Ny grid at one time
// (src/snapshot.cpp:30-80, 405-408): cell (ix, iy) observes at
// O + dX (ix - (Nx-1)/2) + dY (iy - (Ny-1)/2) at time t; integrate() assigns
// the summed retarded field of all particles through
// teufel_cuda_retarded_field.
class SnapshotObserver : public Observer<TrajectorySource> {
public:
    SnapshotObserver(std::string filename, Vector position, Vector dx, Vector dy, unsigned int nx,
                     unsigned int ny, double t)
        : FileName(std::move(filename)), O(position), dX(dx), dY(dy), Nx(nx), Ny(ny), t_obs(t),
          buf(6 * (std::size_t)nx * ny, 0.0) {}
    Vector CellPosition(int ix, int iy) const {
        return O + dX * ((double)ix - 0.5 * ((double)Nx - 1.0)) +
               dY * ((double)iy - 0.5 * ((double)Ny - 1.0));
    }
    void integrate() override {
        if (!source) throw IOexception("SnapshotObserver::integrate - no source set");
        std::vector<double> pos(3 * (std::size_t)Nx * Ny);
        for (unsigned int ix = 0; ix < Nx; ix++)
            for (unsigned int iy = 0; iy < Ny; iy++) {
                const Vector p = CellPosition((int)ix, (int)iy);
                double* q = pos.data() + 3 * ((std::size_t)ix * Ny + iy);
                q[0] = p.x;
                q[1] = p.y;
                q[2] = p.z;
            }
        check_status(teufel_cuda_retarded_field(source->device(), t_obs, (int)(Nx * Ny),
                                                pos.data(), buf.data(), nullptr),
                     "SnapshotObserver::integrate");
    }
    ElMagField getField(unsigned int ix, unsigned int iy) const {
        ElMagField f;
        std::memcpy(f.c, buf.data() + 6 * ((std::size_t)ix * Ny + iy), sizeof f.c);
        return f;
    }
    std::size_t getBufferSize() override { return buf.size(); }
    double* getBuffer() override {
        double* b = new double[buf.size()];
        if (!buf.empty()) std::memcpy(b, buf.data(), sizeof(double) * buf.size());
        return b;
    }
    void fromBuffer(double* buffer, std::size_t size) override {
        if (size != buf.size())
            throw IOexception("SnapshotObserver::fromBuffer() - buffer size mismatch.");
        if (size) std::memcpy(buf.data(), buffer, sizeof(double) * size);
    }
    // Every particle's position and beta*gamma at the snapshot time, kept for
    // the output file (src/snapshot.cpp:114-149); returns the count.
    int storeParticlePositions() {
        particles.clear();
        if (!source) return particlesStored = 0;
        const int nop = source->getNOP();
        particles.resize(6 * (std::size_t)nop);
        for (int i = 0; i < nop; i++) {
            Vector x, bg;
            source->CoordinatesAtTime(i, t_obs, &x, &bg);
            double* q = &particles[6 * (std::size_t)i];
            q[0] = x.x;
            q[1] = x.y;
            q[2] = x.z;
            q[3] = bg.x;
            q[4] = bg.y;
            q[5] = bg.z;
        }
        return particlesStored = nop;
    }
    const std::vector<double>& getParticleCoordinates() const { return particles; }

    // The HDF5 layout of src/snapshot.cpp:226-396: ObservationPosition
    // [Nx][Ny][3] (Nx, Ny), ElMagField [Nx][Ny][6] (t0) and, after
    // storeParticlePositions(), ParticleCoordinates [N][6] (N_particles).
    void WriteFieldHDF5() {
        std::vector<double> pos((std::size_t)Nx * Ny * 3);
        for (unsigned int ix = 0; ix < Nx; ix++)
            for (unsigned int iy = 0; iy < Ny; iy++) {
                const Vector c = CellPosition((int)ix, (int)iy);
                double* q = &pos[((std::size_t)ix * Ny + iy) * 3];
                q[0] = c.x;
                q[1] = c.y;
                q[2] = c.z;
            }
        using h5::AttrOut;
        try {
            h5::Writer w;
            w.add("ObservationPosition", {Nx, Ny, 3}, pos.data(),
                  {AttrOut::Int("Nx", (int32_t)Nx), AttrOut::Int("Ny", (int32_t)Ny)});
            w.add("ElMagField", {Nx, Ny, 6}, buf.data(), {AttrOut::Double("t0", t_obs)});
            if (particlesStored > 0)
                w.add("ParticleCoordinates", {(uint64_t)particlesStored, 6}, particles.data(),
                      {AttrOut::Int("N_particles", particlesStored)});
            w.write(FileName);
        } catch (const h5::Error& e) {
            throw IOexception(std::string("SnapshotObserver::WriteFieldHDF5 - ") + e.what());
        }
    }
    void generateOutput() override { WriteFieldHDF5(); }

private:
    std::string FileName;
    Vector O, dX, dY;
    unsigned int Nx, Ny;
    double t_obs;
    std::vector<double> buf;  // [Nx][Ny][6]
    std::vector<double> particles;  // [particlesStored][6]
    int particlesStored = 0;
};

}  // namespace teufel_gb300
