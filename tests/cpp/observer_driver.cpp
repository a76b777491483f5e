// Exercises the C++ observer layer (include/teufel_observers.hpp) on the GPU:
// reads trajectories and an observer description from a binary file written
// by tests/test_gpu_observers.py, runs ScreenObserver, MeshedScreen and
// PointObserver integrate() and a SnapshotObserver on the same grid at the
// middle of the trace window, and writes their getBuffer() contents; then the
// mesh's buffer after a second integrate() and after zero() + integrate().
//
// input  (doubles unless noted): int32 n_part; int32 npts[n]; charge[n];
//        t[N]; x[N*3]; p[N*3]; a[N*3];
//        origin[3], dx[3], dy[3], int32 nx, int32 ny, t0, dt, dtx, dty, int32 nots
// output: screen buffer [nx*ny*nots*6], mesh buffer (same pixels), point buffer [nots*6],
//         snapshot buffer [nx*ny*6]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "teufel_observers.hpp"

using namespace teufel_gb300;

template <class T>
static void rd(FILE* f, T* p, size_t n) {
    if (fread(p, sizeof(T), n, f) != n) {
        fprintf(stderr, "short read\n");
        exit(2);
    }
}

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    int n = 0;
    rd(f, &n, 1);
    std::vector<int> npts(n);
    rd(f, npts.data(), n);
    std::vector<double> charge(n);
    rd(f, charge.data(), n);
    size_t N = 0;
    for (int v : npts) N += v;
    std::vector<double> t(N), x(3 * N), p(3 * N), a(3 * N);
    rd(f, t.data(), N);
    rd(f, x.data(), 3 * N);
    rd(f, p.data(), 3 * N);
    rd(f, a.data(), 3 * N);
    double o[3], dx[3], dy[3], t0, dt, dtx, dty;
    int nx, ny, nots;
    rd(f, o, 3);
    rd(f, dx, 3);
    rd(f, dy, 3);
    rd(f, &nx, 1);
    rd(f, &ny, 1);
    rd(f, &t0, 1);
    rd(f, &dt, 1);
    rd(f, &dtx, 1);
    rd(f, &dty, 1);
    rd(f, &nots, 1);
    fclose(f);

    TrajectorySource beam;
    size_t off = 0;
    for (int m = 0; m < n; m++) {
        beam.Add(charge[m], npts[m], &t[off], &x[3 * off], &p[3 * off], &a[3 * off]);
        off += npts[m];
    }
    FILE* out = fopen(argv[2], "wb");
    try {
        ScreenObserver scr(Vector(o[0], o[1], o[2]), Vector(dx[0], dx[1], dx[2]),
                           Vector(dy[0], dy[1], dy[2]), nx, ny, t0, dt, dtx, dty, nots);
        scr.setSource(&beam);
        scr.integrate();
        double* b = scr.getBuffer();
        fwrite(b, sizeof(double), scr.getBufferSize(), out);
        delete[] b;
        std::vector<Vector> pts;
        std::vector<double> tz;
        for (int ix = 0; ix < nx; ix++)
            for (int iy = 0; iy < ny; iy++) {
                pts.push_back(scr.CellPosition(ix, iy));
                tz.push_back(scr.CellTimeZero(ix, iy));
            }
        MeshedScreen mesh(pts, tz, dt, nots);
        mesh.setSource(&beam);
        mesh.integrate();
        b = mesh.getBuffer();
        fwrite(b, sizeof(double), mesh.getBufferSize(), out);
        delete[] b;
        const int c = (nx / 2) * ny + ny / 2;
        PointObserver po(pts[c], tz[c], dt, nots);
        po.setSource(&beam);
        po.integrate();
        b = po.getBuffer();
        fwrite(b, sizeof(double), po.getBufferSize(), out);
        delete[] b;
        // a trace shorter than 2 samples: nothing happens, no error
        PointObserver tiny(pts[c], tz[c], dt, 1);
        tiny.setSource(&beam);
        tiny.integrate();
        // the field on the same grid at the middle of the trace window
        SnapshotObserver snap("", Vector(o[0], o[1], o[2]), Vector(dx[0], dx[1], dx[2]),
                              Vector(dy[0], dy[1], dy[2]), nx, ny, t0 + 0.5 * nots * dt);
        snap.setSource(&beam);
        snap.integrate();
        b = snap.getBuffer();
        fwrite(b, sizeof(double), snap.getBufferSize(), out);
        delete[] b;
        // the mesh integrated a second time (added to its traces), then
        // cleared and integrated again (stored)
        mesh.integrate();
        b = mesh.getBuffer();
        fwrite(b, sizeof(double), mesh.getBufferSize(), out);
        delete[] b;
        mesh.zero();
        mesh.integrate();
        b = mesh.getBuffer();
        fwrite(b, sizeof(double), mesh.getBufferSize(), out);
        delete[] b;
    } catch (const IOexception& e) {
        fprintf(stderr, "IOexception: %s\n", e.what());
        fclose(out);
        return 1;
    }
    fclose(out);
    return 0;
}
