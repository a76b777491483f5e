// Drives the C++ observer layer's MeshedScreen / ScreenObserver HDF5 paths
// for tests/test_hdf5.py and tests/test_gpu_diffraction.py.
//
//   mesh_driver read   <file.h5> <out.bin>   MeshedScreen(file) + init(): Np, Nt,
//                                            dt, t0, points, areas, normals, xi,
//                                            eta, total area
//   mesh_driver write  <mesh.bin> <out.h5>   mesh constructor + fromBuffer, init,
//                                            writeFile, read back; prints the
//                                            energies before and after
//   mesh_driver screen <out.h5>              ScreenObserver::generateOutput of a
//                                            fixed 3 x 2 x 4 screen
//   mesh_driver snapshot <parts.bin> <t> <out.h5>
//                                            SnapshotObserver::generateOutput with
//                                            the particles' coordinates at t
//   mesh_driver kat    <mesh.bin> <traj.bin> <in.h5> <out.h5>
//                                            writeFile(in.h5), MeshedScreen(in.h5),
//                                            init, integrate on the GPU from the
//                                            trajectory, totalEnergy, writeFile(out.h5)
//
// mesh.bin: int32 ncp, np, nt; double dt; double corner[ncp][3]; int32
// tri[np][3]; double pos[np][3]; double t0[np]; double field[np][nt][6].
// traj.bin: int32 n; double charge [C]; double t[n], x[n][3], p[n][3], a[n][3].
// parts.bin: int32 count, then count records in the traj.bin format.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "teufel_observers.hpp"

using namespace teufel_gb300;

namespace {

struct Reader {
    std::vector<char> b;
    std::size_t p = 0;
    explicit Reader(const char* path) {
        std::ifstream f(path, std::ios::binary);
        if (!f) throw std::runtime_error(std::string("cannot open ") + path);
        b.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    }
    template <typename T>
    std::vector<T> get(std::size_t n) {
        if (p + n * sizeof(T) > b.size()) throw std::runtime_error("short input");
        std::vector<T> v(n);
        if (n) std::memcpy(v.data(), &b[p], n * sizeof(T));
        p += n * sizeof(T);
        return v;
    }
};

std::vector<Vector> vectors(const std::vector<double>& v) {
    std::vector<Vector> out(v.size() / 3);
    for (std::size_t i = 0; i < out.size(); i++) out[i] = Vector(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    return out;
}

struct Mesh {
    int ncp, np, nt;
    double dt;
    std::vector<double> corner, pos, t0, field;
    std::vector<int32_t> tri;
};

Mesh read_mesh(const char* path) {
    Reader r(path);
    Mesh m;
    const std::vector<int32_t> h = r.get<int32_t>(3);
    m.ncp = h[0];
    m.np = h[1];
    m.nt = h[2];
    m.dt = r.get<double>(1)[0];
    m.corner = r.get<double>(3 * (std::size_t)m.ncp);
    m.tri = r.get<int32_t>(3 * (std::size_t)m.np);
    m.pos = r.get<double>(3 * (std::size_t)m.np);
    m.t0 = r.get<double>((std::size_t)m.np);
    m.field = r.get<double>((std::size_t)m.np * m.nt * 6);
    return m;
}

MeshedScreen* make_screen(const Mesh& m, const std::string& filename) {
    return new MeshedScreen(filename, vectors(m.corner), std::vector<int>(m.tri.begin(), m.tri.end()),
                            vectors(m.pos), m.t0, m.dt, m.nt);
}

void put(std::FILE* f, const void* p, std::size_t n) {
    if (n && std::fwrite(p, 1, n, f) != n) throw std::runtime_error("short write");
}
void put_vec(std::FILE* f, const Vector& v) {
    const double d[3] = {v.x, v.y, v.z};
    put(f, d, sizeof d);
}

int cmd_read(const char* h5, const char* out) {
    MeshedScreen s(h5);
    s.init();
    std::FILE* f = std::fopen(out, "wb");
    if (!f) throw std::runtime_error("cannot create output");
    const int32_t h[2] = {s.get_Np(), s.get_Nt()};
    put(f, h, sizeof h);
    const double dt = s.get_dt(), area = s.getTotalArea();
    put(f, &dt, 8);
    put(f, &area, 8);
    for (int i = 0; i < s.get_Np(); i++) {
        const double t0 = s.get_t0(i), a = s.get_area(i);
        put(f, &t0, 8);
        put_vec(f, s.get_point(i));
        put(f, &a, 8);
        put_vec(f, s.get_normal(i));
        put_vec(f, s.get_xi(i));
        put_vec(f, s.get_eta(i));
    }
    std::fclose(f);
    return 0;
}

int cmd_write(const char* in, const char* h5) {
    const Mesh m = read_mesh(in);
    MeshedScreen* s = make_screen(m, h5);
    std::vector<double> f = m.field;
    s->fromBuffer(f.data(), f.size());
    s->init();
    const double e1 = s->totalEnergy();
    s->generateOutput();  // writeFile(FileName)
    MeshedScreen back(h5);
    back.init();
    const double e2 = back.totalEnergy();
    double* b1 = s->getBuffer();
    double* b2 = back.getBuffer();
    const bool same = s->getBufferSize() == back.getBufferSize() &&
                      std::memcmp(b1, b2, sizeof(double) * s->getBufferSize()) == 0;
    delete[] b1;
    delete[] b2;
    std::printf("energy %.17g %.17g buffer %s\n", e1, e2, same ? "same" : "different");
    delete s;
    return same ? 0 : 1;
}

int cmd_screen(const char* h5) {
    ScreenObserver scr(h5, Vector(0.001, -0.002, 2.5), Vector(0.01, 0.0, 0.0), Vector(0.0, 0.02, 0.0),
                       3, 2, 8.3e-9, 1e-13, 2e-14, -3e-14, 4);
    std::vector<double> f(scr.getBufferSize());
    for (std::size_t i = 0; i < f.size(); i++) f[i] = 0.25 * (double)i - 7.0;
    scr.fromBuffer(f.data(), f.size());
    scr.generateOutput();
    return 0;
}

// traj.bin particles (trajectory format above, n points each, count given by
// the file), a 4 x 3 snapshot at time t with ramp fields, particle coordinates
// stored, written by generateOutput().
int cmd_snapshot(const char* traj, double t, const char* h5) {
    Reader r(traj);
    const int nop = r.get<int32_t>(1)[0];
    TrajectorySource src;
    for (int m = 0; m < nop; m++) {
        const int n = r.get<int32_t>(1)[0];
        const double charge = r.get<double>(1)[0];
        const std::vector<double> tt = r.get<double>((std::size_t)n), x = r.get<double>(3 * (std::size_t)n),
                                  p = r.get<double>(3 * (std::size_t)n), a = r.get<double>(3 * (std::size_t)n);
        src.Add(charge, n, tt.data(), x.data(), p.data(), a.data());
    }
    SnapshotObserver snap(h5, Vector(0.0, 0.1, 3.0), Vector(0.002, 0.0, 0.0), Vector(0.0, 0.003, 0.0),
                          4, 3, t);
    snap.setSource(&src);
    std::vector<double> f(snap.getBufferSize());
    for (std::size_t i = 0; i < f.size(); i++) f[i] = 1.5 * (double)i + 0.25;
    snap.fromBuffer(f.data(), f.size());
    const int stored = snap.storeParticlePositions();
    snap.generateOutput();
    std::printf("stored %d\n", stored);
    return 0;
}

int cmd_kat(const char* in, const char* traj, const char* h5_in, const char* h5_out) {
    const Mesh m = read_mesh(in);
    {
        MeshedScreen* s = make_screen(m, h5_in);
        s->writeFile();
        delete s;
    }
    Reader r(traj);
    const int n = r.get<int32_t>(1)[0];
    const double charge = r.get<double>(1)[0];
    const std::vector<double> t = r.get<double>((std::size_t)n), x = r.get<double>(3 * (std::size_t)n),
                              p = r.get<double>(3 * (std::size_t)n), a = r.get<double>(3 * (std::size_t)n);
    TrajectorySource bunch;
    bunch.Add(charge, n, t.data(), x.data(), p.data(), a.data());
    // the reference's test body, tests/teufel.DiffractionScreen.cpp:134-147
    MeshedScreen screen(h5_in);
    screen.init();
    screen.zero();
    screen.setSource(&bunch);
    screen.integrate();
    const double EuJ = screen.totalEnergy() * 1.0e6;
    screen.writeFile(h5_out);
    std::printf("energy_uJ %.17g\n", EuJ);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    try {
        const std::string c = argc > 1 ? argv[1] : "";
        if (c == "read" && argc == 4) return cmd_read(argv[2], argv[3]);
        if (c == "write" && argc == 4) return cmd_write(argv[2], argv[3]);
        if (c == "screen" && argc == 3) return cmd_screen(argv[2]);
        if (c == "snapshot" && argc == 5) return cmd_snapshot(argv[2], std::atof(argv[3]), argv[4]);
        if (c == "kat" && argc == 6) return cmd_kat(argv[2], argv[3], argv[4], argv[5]);
        std::fprintf(stderr, "usage: mesh_driver read|write|screen|kat ...\n");
        return 2;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 3;
    }
}
