// lattice.cpp -- the createLattice geometry (src/object.cu:232-293): masses
// in i, j, k order at ((i/(nx-1) - 0.5) * dims + center), springs to the 13
// forward neighbours of the 26-neighbourhood in the builder's loop order
// (this order is the spring numbering users see, so it is kept), rest
// length = |right - left|.
#include <cmath>
#include <cstdint>

#include "titan_gb300.h"

namespace {

struct Emit {
    int32_t *left, *right;
    int64_t count = 0;
    void operator()(int32_t l, int32_t r) {
        if (left) left[count] = l;
        if (right) right[count] = r;
        count++;
    }
};

template <typename F>
void lattice_springs(int nx, int ny, int nz, F &&emit) {
    auto id = [&](int i, int j, int k) { return (int32_t)(k + j * nz + i * ny * nz); };
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                const bool ei = i != nx - 1, ej = j != ny - 1, ek = k != nz - 1;
                for (int l = 0; l <= (ei ? 1 : 0); l++)
                    for (int m = 0; m <= (ej ? 1 : 0); m++)
                        for (int n = 0; n <= (ek ? 1 : 0); n++)
                            if (l || m || n) emit(id(i, j, k), id(i + l, j + m, k + n));
                if (ek) {
                    if (ej) emit(id(i, j, k + 1), id(i, j + 1, k));
                    if (ei) emit(id(i, j, k + 1), id(i + 1, j, k));
                    if (ej && ei) {
                        emit(id(i, j, k + 1), id(i + 1, j + 1, k));
                        emit(id(i + 1, j, k + 1), id(i, j + 1, k));
                        emit(id(i, j + 1, k + 1), id(i + 1, j, k));
                    }
                }
                if (ej && ei) emit(id(i, j + 1, k), id(i + 1, j, k));
            }
}

}  // namespace

extern "C" int64_t titan_gb300_lattice_springs(int nx, int ny, int nz) {
    if (nx <= 0 || ny <= 0 || nz <= 0) return 0;
    Emit e{nullptr, nullptr};
    lattice_springs(nx, ny, nz, e);
    return e.count;
}

extern "C" int titan_gb300_lattice(const double center[3], const double dims[3], int nx, int ny, int nz,
                                   double *pos, int32_t *left, int32_t *right, double *rest) {
    if (!center || !dims || !pos || nx <= 0 || ny <= 0 || nz <= 0) return TITAN_GB300_EINVAL;
    int64_t q = 0;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
                double u = (nx > 1) ? (double)i / (nx - 1.0) - 0.5 : 0;
                double v = (ny > 1) ? j / (ny - 1.0) - 0.5 : 0;
                double w = (nz > 1) ? k / (nz - 1.0) - 0.5 : 0;
                pos[3 * q] = u * dims[0] + center[0];
                pos[3 * q + 1] = v * dims[1] + center[1];
                pos[3 * q + 2] = w * dims[2] + center[2];
                q++;
            }
    if (!left && !right && !rest) return TITAN_GB300_OK;
    Emit e{left, right};
    lattice_springs(nx, ny, nz, e);
    if (rest && left && right)
        for (int64_t s = 0; s < e.count; s++) {
            const double *a = pos + 3 * left[s], *b = pos + 3 * right[s];
            double d0 = b[0] - a[0], d1 = b[1] - a[1], d2 = b[2] - a[2];
            double x = d0 * d0, y = d1 * d1, z = d2 * d2;
            rest[s] = std::sqrt((x + y) + z);
        }
    return TITAN_GB300_OK;
}
