// Writes a PointObserver trace through the C++ observer layer's SDDS writer
// (no GPU involved): the trace comes from a binary file via fromBuffer().
//   sdds_driver <in.bin> <out.sdds>
//   in.bin: double t0, double dt, int32 N, double f[N][6]
#include <cstdint>
#include <cstdio>
#include <vector>

#include "teufel_observers.hpp"

using namespace teufel_gb300;

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    std::FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    double t0 = 0.0, dt = 0.0;
    int32_t n = 0;
    if (std::fread(&t0, sizeof t0, 1, f) != 1 || std::fread(&dt, sizeof dt, 1, f) != 1 ||
        std::fread(&n, sizeof n, 1, f) != 1 || n < 0)
        return 4;
    std::vector<double> buf(6 * (size_t)n);
    if (n && std::fread(buf.data(), sizeof(double), buf.size(), f) != buf.size()) return 5;
    std::fclose(f);
    try {
        PointObserver obs(argv[2], Vector(0.0, 0.0, 1.0), t0, dt, (std::size_t)n);
        obs.fromBuffer(buf.data(), buf.size());
        obs.generateOutput();
    } catch (const IOexception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
