// Host-only mesh utilities of the C ABI: the hexahedral grid generator with
// five tets per hex (the reference's MeshUtils::createBeamMsh,
// src/utils/MeshUtils.cpp:424-660) and its surface triangulation.
#include <cstdint>

#include "../../include/xpbd_gpu.h"

namespace {

struct Grid {
    int nx, ny, nz;  // hexes along x (width), y (length), z (height)
    int64_t vid(int ix, int iy, int iz) const {
        // reference order: height fastest, then width, then length
        return (int64_t)iz + (int64_t)ix * (nz + 1) + (int64_t)iy * (nx + 1) * (nz + 1);
    }
};

// Two triangles of a boundary quad with corners (a, b, c, d) in cyclic order,
// split along a-c (first) or b-d (second). `flip` reverses the winding.
void quad(int32_t*& out, int64_t a, int64_t b, int64_t c, int64_t d, bool diag_ac, bool flip) {
    int64_t t[6];
    if (diag_ac) { t[0] = a; t[1] = b; t[2] = c; t[3] = a; t[4] = c; t[5] = d; }
    else         { t[0] = a; t[1] = b; t[2] = d; t[3] = b; t[4] = c; t[5] = d; }
    if (flip) { int64_t s = t[1]; t[1] = t[2]; t[2] = s; s = t[4]; t[4] = t[5]; t[5] = s; }
    for (int k = 0; k < 6; k++) *out++ = (int32_t)t[k];
}

}  // namespace

extern "C" {

int xpbd_grid_counts(int32_t nx, int32_t ny, int32_t nz, int64_t* nv, int64_t* nt, int64_t* nf) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || !nv || !nt || !nf) return XPBD_ERR_INVALID;
    *nv = (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
    *nt = 5LL * nx * ny * nz;
    *nf = 4LL * ((int64_t)nx * nz + (int64_t)ny * nz + (int64_t)nx * ny);
    return XPBD_OK;
}

int xpbd_grid_mesh(int32_t nx, int32_t ny, int32_t nz, double hx, double hy, double hz, int32_t split, double* X,
                   int32_t* tets, int32_t* faces) {
    if (nx <= 0 || ny <= 0 || nz <= 0 || !X || !tets || !faces || (split != 0 && split != 1)) return XPBD_ERR_INVALID;
    const Grid g{nx, ny, nz};
    const bool uniform = split == 1;
    for (int iy = 0; iy <= ny; iy++)
        for (int ix = 0; ix <= nx; ix++)
            for (int iz = 0; iz <= nz; iz++) {
                const int64_t v = g.vid(ix, iy, iz);
                X[3 * v] = ix * hx;
                X[3 * v + 1] = iy * hy;
                X[3 * v + 2] = iz * hz;
            }
    // Surface: y = 0 / y = ny quads, then x = nx / x = 0, then z = nz / z = 0,
    // in the reference's emission order. Diagonal choice: the alternating
    // checkerboard of the current generator, or (split = 1) the rule of the
    // revision that wrote the reference's cube2/cube4 fixtures.
    int32_t* f = faces;
    for (int ix = 0; ix < nx; ix++)
        for (int iz = 0; iz < nz; iz++) {
            const bool eq = (ix & 1) == (iz & 1);
            bool ac = uniform ? !eq : eq;
            quad(f, g.vid(ix, 0, iz), g.vid(ix + 1, 0, iz), g.vid(ix + 1, 0, iz + 1), g.vid(ix, 0, iz + 1), ac, false);
            ac = uniform ? !eq : (eq != ((ny & 1) != 0));
            quad(f, g.vid(ix, ny, iz), g.vid(ix + 1, ny, iz), g.vid(ix + 1, ny, iz + 1), g.vid(ix, ny, iz + 1), ac,
                 true);
        }
    for (int iz = 0; iz < nz; iz++)
        for (int iy = 0; iy < ny; iy++) {
            const bool eq = (iz & 1) == (iy & 1);
            bool ac = uniform ? !eq : (eq != ((nx & 1) != 0));
            quad(f, g.vid(nx, iy, iz), g.vid(nx, iy + 1, iz), g.vid(nx, iy + 1, iz + 1), g.vid(nx, iy, iz + 1), ac,
                 false);
            ac = uniform ? !eq : eq;
            quad(f, g.vid(0, iy, iz), g.vid(0, iy + 1, iz), g.vid(0, iy + 1, iz + 1), g.vid(0, iy, iz + 1), ac, true);
        }
    for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nx; ix++) {
            const bool eq = (iy & 1) == (ix & 1);
            bool ac = uniform ? !eq : (eq != ((nz & 1) != 0));
            quad(f, g.vid(ix, iy, nz), g.vid(ix + 1, iy, nz), g.vid(ix + 1, iy + 1, nz), g.vid(ix, iy + 1, nz), ac,
                 false);
            ac = uniform ? !eq : eq;
            quad(f, g.vid(ix, iy, 0), g.vid(ix + 1, iy, 0), g.vid(ix + 1, iy + 1, 0), g.vid(ix, iy + 1, 0), ac, true);
        }
    // Five tets per hex. Corners c[0..7] = (x,y,z) offsets (000,100,110,010,001,101,111,011);
    // pattern A keeps corners 0,2,5,7 as the central tet, pattern B corners 1,3,4,6.
    static const int A[5][4] = {{0, 1, 2, 5}, {0, 2, 3, 7}, {0, 5, 4, 7}, {2, 5, 6, 7}, {0, 2, 5, 7}};
    static const int B[5][4] = {{0, 3, 1, 4}, {1, 3, 2, 6}, {1, 5, 4, 6}, {3, 4, 7, 6}, {1, 3, 4, 6}};
    int32_t* t = tets;
    for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nx; ix++)
            for (int iz = 0; iz < nz; iz++) {
                const int64_t c[8] = {g.vid(ix, iy, iz),         g.vid(ix + 1, iy, iz),     g.vid(ix + 1, iy + 1, iz),
                                      g.vid(ix, iy + 1, iz),     g.vid(ix, iy, iz + 1),     g.vid(ix + 1, iy, iz + 1),
                                      g.vid(ix + 1, iy + 1, iz + 1), g.vid(ix, iy + 1, iz + 1)};
                // selector (hz%2 == hx%2) - hy%2, nonzero (including -1) picks A
                const int sel = (int)((iz & 1) == (ix & 1)) - (iy & 1);
                const int(*P)[4] = (uniform || sel != 0) ? A : B;
                for (int k = 0; k < 5; k++)
                    for (int j = 0; j < 4; j++) *t++ = (int32_t)c[P[k][j]];
            }
    return XPBD_OK;
}

}  // extern "C"
