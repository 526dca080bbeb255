// ORACLE — test infrastructure only.  A CPU restatement of the reference MR-LBM D3Q27 time
// step (sakthi-lbm/MRLBM_3D_CUDA), used by tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py to check the CUDA solver.  It is never linked into or called
// by the product library.
//
// Written to follow the reference literally rather than fast: the populations are rebuilt
// into a full array and pulled with a periodic wrap in every axis (equivalent to the
// reference's block-local streaming plus halo faces), every closure keeps the reference's
// expression order, and T = float reproduces the reference's FP32 rounding while
// T = double gives the FP64 run.  Paths below are inside the reference repository:
//   lattice tables            MRLBM_3D/src/core/D3Q27/latticeProperties.cuh:5-31
//   pop_reconstruction        MRLBM_3D/src/core/D3Q27/second_order/reconstruction.cuh:5-60
//   evaluate_moments          MRLBM_3D/src/core/D3Q27/eval_moments.cuh:5-22
//   moment_collision          MRLBM_3D/src/solver/mlbm.cu:3-16
//   kernel A / kernel B       MRLBM_3D/src/solver/mlbm.cu:83-164, 186-242
//   step order                MRLBM_3D/src/main.cu:21-35
//   planar closures           MRLBM_3D/src/cases/cylinder/boundaries.cuh:8-843
//   BCFLUID closure           MRLBM_3D/src/cases/cylinder/boundaries.cuh:845-1037
//   BCSOLID closure           MRLBM_3D/src/cases/cylinder/boundaries.cuh:1039-1214 (z walls only)
//   curved-wall closure       MRLBM_3D/src/boundary/curvedLBM.cu:5-132, extrapolation_utils.cuh:5-107,
//                             numerical_solution.cu:4-279
//   forces                    MRLBM_3D/src/statistics/forces.cu:3-133
//   initialiser               MRLBM_3D/src/solver/initializeLBM.cu:24-121
//   geometry                  MRLBM_3D/src/cases/{cylinder,annulus}/nodeClass.cuh, cylinder_helpers.cuh
//   active blocks             MRLBM_3D/src/simulation.cu:174-214, solver/mlbm.cu:87-89
// Build: g++ -O2 -fopenmp -ffp-contract=off -shared -fPIC (oracle/build_oracle.py).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../include/mrlbm.h"

namespace {

const int CX[27] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1};
const int CY[27] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1};
const int CZ[27] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1};
const int OPP[27] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17, 20, 19, 22, 21, 24, 23, 26, 25};
// octant bit b -> its 7 directions (nodeClass.cuh:67-75)
const int OCT[8][7] = {{2, 4, 6, 8, 10, 12, 20}, {1, 4, 6, 12, 13, 15, 26}, {2, 3, 6, 10, 14, 17, 24},
                       {1, 3, 6, 7, 15, 17, 21}, {2, 4, 5, 8, 16, 18, 22}, {1, 4, 5, 9, 13, 18, 23},
                       {2, 3, 5, 11, 14, 16, 25}, {1, 3, 5, 7, 9, 11, 19}};

enum : uint32_t {
    BULK = 0, SOLID, INNER, OUTER, BCF_IN, BCF_OUT, BCS_IN, BCS_OUT,
    NORTH, SOUTH, EAST, WEST, FRONT, BACK,
    NORTH_EAST, NORTH_WEST, NORTH_FRONT, NORTH_BACK, SOUTH_EAST, SOUTH_WEST, SOUTH_FRONT, SOUTH_BACK,
    EAST_FRONT, EAST_BACK, WEST_FRONT, WEST_BACK,
    NWF, NWB, SWF, SWB, NEF, NEB, SEF, SEB
};

std::string g_err;

// All fixed-point constants of the reference are `real` (float) constexprs; the arithmetic
// type T decides the rest.
template <typename T>
struct Lat {
    T w[27], cs2, as2;
    T hxx[27], hyy[27], hzz[27], hxy[27], hxz[27], hyz[27];
    Lat() {
        const float W0 = (float)(8.0 / 27.0), W1 = (float)(2.0 / 27.0), W2 = (float)(1.0 / 54.0), W3 = (float)(1.0 / 216.0);
        for (int q = 0; q < 27; ++q) w[q] = q == 0 ? W0 : q <= 6 ? W1 : q <= 18 ? W2 : W3;
        as2 = (T)3.0f;
        cs2 = std::is_same<T, float>::value ? (T)(float)(1.0 / 3.0) : (T)(1.0 / 3.0);
        if (std::is_same<T, double>::value) {
            w[0] = 8.0 / 27.0;
            for (int q = 1; q < 27; ++q) w[q] = q <= 6 ? 2.0 / 27.0 : q <= 18 ? 1.0 / 54.0 : 1.0 / 216.0;
        }
        for (int q = 0; q < 27; ++q) {
            hxx[q] = (T)CX[q] * (T)CX[q] - cs2;
            hyy[q] = (T)CY[q] * (T)CY[q] - cs2;
            hzz[q] = (T)CZ[q] * (T)CZ[q] - cs2;
            hxy[q] = (T)CX[q] * (T)CY[q];
            hxz[q] = (T)CX[q] * (T)CZ[q];
            hyz[q] = (T)CY[q] * (T)CZ[q];
        }
    }
};

template <typename T>
struct M10 {
    T rho, ux, uy, uz, mxx, myy, mzz, mxy, mxz, myz;
};

template <typename T>
void reconstruct(const Lat<T> &L, const M10<T> &m, T *pop) {
    const T rho = m.rho * (T)1.0f;
    const T ux = m.ux * L.as2, uy = m.uy * L.as2, uz = m.uz * L.as2;
    const T s2 = (T)0.5f * L.as2 * L.as2, s11 = L.as2 * L.as2;
    const T mxx = m.mxx * s2, myy = m.myy * s2, mzz = m.mzz * s2;
    const T mxy = m.mxy * s11, mxz = m.mxz * s11, myz = m.myz * s11;
    const T mtrace = mxx + myy + mzz;
    T mt = rho * L.w[0];
    const T pics2 = (T)1.0f - L.cs2 * mtrace;
    pop[0] = mt * (pics2);
    mt = rho * L.w[1];
    pop[1] = mt * (pics2 + ux + mxx);
    pop[2] = mt * (pics2 - ux + mxx);
    pop[3] = mt * (pics2 + uy + myy);
    pop[4] = mt * (pics2 - uy + myy);
    pop[5] = mt * (pics2 + uz + mzz);
    pop[6] = mt * (pics2 - uz + mzz);
    mt = rho * L.w[7];
    pop[7] = mt * (pics2 + ux + uy + mxx + myy + mxy);
    pop[8] = mt * (pics2 - ux - uy + mxx + myy + mxy);
    pop[9] = mt * (pics2 + ux + uz + mxx + mzz + mxz);
    pop[10] = mt * (pics2 - ux - uz + mxx + mzz + mxz);
    pop[11] = mt * (pics2 + uy + uz + myy + mzz + myz);
    pop[12] = mt * (pics2 - uy - uz + myy + mzz + myz);
    pop[13] = mt * (pics2 + ux - uy + mxx + myy - mxy);
    pop[14] = mt * (pics2 - ux + uy + mxx + myy - mxy);
    pop[15] = mt * (pics2 + ux - uz + mxx + mzz - mxz);
    pop[16] = mt * (pics2 - ux + uz + mxx + mzz - mxz);
    pop[17] = mt * (pics2 + uy - uz + myy + mzz - myz);
    pop[18] = mt * (pics2 - uy + uz + myy + mzz - myz);
    mt = rho * L.w[19];
    pop[19] = mt * (pics2 + ux + uy + uz + mtrace + (mxy + mxz + myz));
    pop[20] = mt * (pics2 - ux - uy - uz + mtrace + (mxy + mxz + myz));
    pop[21] = mt * (pics2 + ux + uy - uz + mtrace + (mxy - mxz - myz));
    pop[22] = mt * (pics2 - ux - uy + uz + mtrace + (mxy - mxz - myz));
    pop[23] = mt * (pics2 + ux - uy + uz + mtrace - (mxy - mxz + myz));
    pop[24] = mt * (pics2 - ux + uy - uz + mtrace - (mxy - mxz + myz));
    pop[25] = mt * (pics2 - ux + uy + uz + mtrace - (mxy + mxz - myz));
    pop[26] = mt * (pics2 + ux - uy - uz + mtrace - (mxy + mxz - myz));
}

template <typename T>
void evaluate(const Lat<T> &L, const T *p, M10<T> &m) {
    m.rho = p[0] + p[1] + p[2] + p[3] + p[4] + p[5] + p[6] + p[7] + p[8] + p[9] + p[10] + p[11] + p[12] + p[13] + p[14] +
            p[15] + p[16] + p[17] + p[18] + p[19] + p[20] + p[21] + p[22] + p[23] + p[24] + p[25] + p[26];
    const T inv = (T)1 / m.rho;
    m.ux = ((p[1] + p[7] + p[9] + p[13] + p[15] + p[19] + p[21] + p[23] + p[26]) -
            (p[2] + p[8] + p[10] + p[14] + p[16] + p[20] + p[22] + p[24] + p[25])) * inv;
    m.uy = ((p[3] + p[7] + p[11] + p[14] + p[17] + p[19] + p[21] + p[24] + p[25]) -
            (p[4] + p[8] + p[12] + p[13] + p[18] + p[20] + p[22] + p[23] + p[26])) * inv;
    m.uz = ((p[5] + p[9] + p[11] + p[16] + p[18] + p[19] + p[22] + p[23] + p[25]) -
            (p[6] + p[10] + p[12] + p[15] + p[17] + p[20] + p[21] + p[24] + p[26])) * inv;
    m.mxx = (p[1] + p[2] + p[7] + p[8] + p[9] + p[10] + p[13] + p[14] + p[15] + p[16] + p[19] + p[20] + p[21] + p[22] +
             p[23] + p[24] + p[25] + p[26]) * inv - L.cs2;
    m.myy = (p[3] + p[4] + p[7] + p[8] + p[11] + p[12] + p[13] + p[14] + p[17] + p[18] + p[19] + p[20] + p[21] + p[22] +
             p[23] + p[24] + p[25] + p[26]) * inv - L.cs2;
    m.mzz = (p[5] + p[6] + p[9] + p[10] + p[11] + p[12] + p[15] + p[16] + p[17] + p[18] + p[19] + p[20] + p[21] + p[22] +
             p[23] + p[24] + p[25] + p[26]) * inv - L.cs2;
    m.mxy = ((p[7] + p[8] + p[19] + p[20] + p[21] + p[22]) - (p[13] + p[14] + p[23] + p[24] + p[25] + p[26])) * inv;
    m.mxz = ((p[9] + p[10] + p[19] + p[20] + p[23] + p[24]) - (p[15] + p[16] + p[21] + p[22] + p[25] + p[26])) * inv;
    m.myz = ((p[11] + p[12] + p[19] + p[20] + p[25] + p[26]) - (p[17] + p[18] + p[21] + p[22] + p[23] + p[24])) * inv;
}

template <typename T>
void collide(T omega, M10<T> &m) {
    const T om1 = (T)1.0f - omega;
    m.mxx = om1 * m.mxx + omega * m.ux * m.ux;
    m.myy = om1 * m.myy + omega * m.uy * m.uy;
    m.mzz = om1 * m.mzz + omega * m.uz * m.uz;
    m.mxy = om1 * m.mxy + omega * m.ux * m.uy;
    m.mxz = om1 * m.mxz + omega * m.ux * m.uz;
    m.myz = om1 * m.myz + omega * m.uy * m.uz;
}

struct WallO {
    std::vector<int64_t> list, fluid, solid;
    std::vector<float> nx, ny, delta;
    std::vector<uint32_t> in, out;
};

template <typename T>
struct Oracle {
    mrlbm_case_desc d;
    Lat<T> L;
    int nx, ny, nz;
    int64_t n;
    T omega, rho0, umax;
    std::vector<uint32_t> type;  // reference encoding: class << 20 | index
    std::vector<uint8_t> frozen;
    WallO wall[2];
    int n_walls = 0;
    uint32_t tag_in[256] = {0}, tag_out[256] = {0};
    std::vector<T> mom[10];     // post-collision moments, rho stored as rho - rho0
    std::vector<T> pops;        // 27 x n work array
    int64_t step = 0;
    double force[10] = {0};

    int64_t idx(int x, int y, int z) const { return x + (int64_t)nx * (y + (int64_t)ny * z); }
    uint32_t cls(int64_t i) const { return type[i] >> 20; }

    M10<T> load(int64_t i) const {
        M10<T> m;
        m.rho = rho0 + mom[0][i];
        m.ux = mom[1][i]; m.uy = mom[2][i]; m.uz = mom[3][i];
        m.mxx = mom[4][i]; m.myy = mom[5][i]; m.mzz = mom[6][i];
        m.mxy = mom[7][i]; m.mxz = mom[8][i]; m.myz = mom[9][i];
        return m;
    }
    void store(int64_t i, const M10<T> &m) {
        mom[0][i] = m.rho - rho0;
        mom[1][i] = m.ux; mom[2][i] = m.uy; mom[3][i] = m.uz;
        mom[4][i] = m.mxx; mom[5][i] = m.myy; mom[6][i] = m.mzz;
        mom[7][i] = m.mxy; mom[8][i] = m.mxz; mom[9][i] = m.myz;
    }

    // ---------------- geometry (restated from the reference host code) -------------------
    uint32_t face(int x, int y, int z) const {
        bool W = x == 0, E = x == nx - 1, S = y == 0, N = y == ny - 1, B = z == 0, F = z == nz - 1;
        if (d.periodic[0]) W = E = false;
        if (d.periodic[1]) S = N = false;
        if (d.periodic[2]) B = F = false;
        if (N && W && F) return NWF;
        if (N && W && B) return NWB;
        if (N && E && F) return NEF;
        if (N && E && B) return NEB;
        if (S && W && F) return SWF;
        if (S && W && B) return SWB;
        if (S && E && F) return SEF;
        if (S && E && B) return SEB;
        if (N && W) return NORTH_WEST;
        if (N && E) return NORTH_EAST;
        if (N && F) return NORTH_FRONT;
        if (N && B) return NORTH_BACK;
        if (S && W) return SOUTH_WEST;
        if (S && E) return SOUTH_EAST;
        if (S && F) return SOUTH_FRONT;
        if (S && B) return SOUTH_BACK;
        if (W && F) return WEST_FRONT;
        if (W && B) return WEST_BACK;
        if (E && F) return EAST_FRONT;
        if (E && B) return EAST_BACK;
        if (N) return NORTH;
        if (S) return SOUTH;
        if (W) return WEST;
        if (E) return EAST;
        if (F) return FRONT;
        if (B) return BACK;
        return BULK;
    }
    void neighbours(int x, int y, int z, uint32_t *nb) const {
        for (int q = 0; q < 27; ++q) {
            int xn = x + CX[q], yn = y + CY[q], zn = z + CZ[q];
            bool out;
            if (d.periodic[2]) {
                zn = zn < 0 ? zn + nz : (zn >= nz ? zn - nz : zn);
                out = xn < 0 || xn >= nx || yn < 0 || yn >= ny;
            } else {
                out = xn < 0 || xn >= nx || yn < 0 || yn >= ny || zn < 0 || zn >= nz;
            }
            nb[q] = out ? SOLID : cls(idx(xn, yn, zn));
        }
    }
    int bits_of(const uint32_t *nb, uint32_t t, int *bits) const {
        int c = 0;
        for (int b = 0; b < 8; ++b) {
            bits[b] = 0;
            for (int k = 0; k < 7; ++k)
                if (nb[OCT[b][k]] == t) { bits[b] = 1; break; }
            c += bits[b];
        }
        return c;
    }
    std::string geometry() {
        type.assign(n, 0);
        frozen.assign(n, 0);
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x) type[idx(x, y, z)] = face(x, y, z) << 20;
        n_walls = d.geometry == MRLBM_GEOM_CYLINDER ? 1 : d.geometry == MRLBM_GEOM_ANNULUS ? 2 : 0;
        if (n_walls) {
            const float XC = d.xc, YC = d.yc;
            const float RIN = 0.5f * d.d_wall[0], ROUT = 0.5f * d.d_wall[1];
            const float RMID = (float)(0.5 * (double)(float)(RIN + ROUT));
            auto radius = [&](int x, int y) {
                const float a = (float)x - XC, b = (float)y - YC;
                return std::sqrt(a * a + b * b);
            };
            for (int z = 0; z < nz; ++z)
                for (int y = 0; y < ny; ++y)
                    for (int x = 0; x < nx; ++x) {
                        const float r = radius(x, y);
                        const bool s = n_walls == 1 ? r <= RIN : (r <= RIN || r >= ROUT);
                        if (s) type[idx(x, y, z)] = SOLID << 20;
                    }
            const int Z0 = d.periodic[2] ? 0 : 1, Z1 = d.periodic[2] ? nz : nz - 1;
            uint32_t nb[27];
            int bits[8];
            for (int z = Z0; z < Z1; ++z)
                for (int y = d.scan_box[2]; y < d.scan_box[3]; ++y)
                    for (int x = d.scan_box[0]; x < d.scan_box[1]; ++x) {
                        neighbours(x, y, z, nb);
                        bool fluid = false;
                        for (int q = 1; q < 27; ++q) fluid = fluid || nb[q] == BULK;
                        if (!(nb[0] == SOLID && fluid)) continue;
                        bool take = true;
                        if (d.triangular) {
                            const int c = bits_of(nb, BULK, bits);
                            take = d.periodic[2] ? c > 2 : (((z == 0 || z == nz - 1) && c > 1) || (z > 0 && z < nz - 1 && c > 2));
                        }
                        if (take) type[idx(x, y, z)] = ((n_walls == 2 && !(radius(x, y) < RMID)) ? OUTER : INNER) << 20;
                    }
            if (d.triangular)
                for (int z = Z0; z < Z1; ++z)
                    for (int y = d.scan_box[2]; y < d.scan_box[3]; ++y)
                        for (int x = d.scan_box[0]; x < d.scan_box[1]; ++x) {
                            neighbours(x, y, z, nb);
                            bool solid = false;
                            for (int q = 1; q < 27; ++q) solid = solid || nb[q] == SOLID;
                            if (!(nb[0] == BULK && solid)) continue;
                            bits_of(nb, SOLID, bits);
                            uint32_t tag = 0;
                            for (int b = 0; b < 8; ++b) tag += (uint32_t)bits[b] << b;
                            const uint32_t c = (n_walls == 2 && !(radius(x, y) < RMID)) ? BCF_OUT : BCF_IN;
                            type[idx(x, y, z)] = (c << 20) | tag;
                        }
            // BCSOLID (nodeClass.cuh:254-287, annulus/nodeClass.cuh:309-357): z walls only
            if (d.triangular && !d.periodic[2])
                for (int z : {0, nz - 1})
                    for (int y = d.scan_box[2]; y < d.scan_box[3]; ++y)
                        for (int x = d.scan_box[0]; x < d.scan_box[1]; ++x) {
                            neighbours(x, y, z, nb);
                            if (nb[0] != BACK && nb[0] != FRONT) continue;
                            if (bits_of(nb, BULK, bits) >= 4) continue;
                            uint32_t tag = 0;
                            for (int b = 0; b < 8; ++b) tag += (uint32_t)bits[b] << b;
                            const uint32_t c = (n_walls == 2 && !(radius(x, y) < RMID)) ? BCS_OUT : BCS_IN;
                            type[idx(x, y, z)] = (c << 20) | tag;
                        }
            for (int64_t i = 0; i < n; ++i) {
                const uint32_t c = cls(i);
                if (c == INNER) wall[0].list.push_back(i);
                else if (c == OUTER) wall[1].list.push_back(i);
                else if (c == BCF_IN) wall[0].fluid.push_back(i);
                else if (c == BCF_OUT) wall[1].fluid.push_back(i);
                else if (c == BCS_IN) wall[0].solid.push_back(i);
                else if (c == BCS_OUT) wall[1].solid.push_back(i);
            }
            for (int w = 0; w < n_walls; ++w) {
                WallO &W = wall[w];
                const float rw = 0.5f * d.d_wall[w];
                for (size_t i = 0; i < W.list.size(); ++i) {
                    const int64_t g = W.list[i];
                    type[g] = (type[g] & 0xFFF00000u) | (uint32_t)i;
                    const int x = (int)(g % nx), y = (int)((g / nx) % ny), z = (int)(g / ((int64_t)nx * ny));
                    const float xb = (float)x, yb = (float)y;
                    const float dx = xb - XC, dy = yb - YC;
                    const float r2 = dx * dx + dy * dy;
                    const float inv = (float)(1.0 / std::sqrt((double)r2));
                    const float ux = dx * inv, uy = dy * inv;
                    const float xw = XC + rw * ux, yw = YC + rw * uy;
                    W.nx.push_back(ux);
                    W.ny.push_back(uy);
                    W.delta.push_back(std::fabs((xw - xb) * ux + (yw - yb) * uy));
                    neighbours(x, y, z, nb);
                    uint32_t in = 1u;
                    for (int b = 0; b < 8; ++b) {
                        bool ok = true;
                        for (int k = 0; k < 7; ++k) ok = ok && nb[OCT[b][k]] != SOLID;
                        if (ok)
                            for (int k = 0; k < 7; ++k) in |= 1u << OPP[OCT[b][k]];
                    }
                    uint32_t out = 1u;
                    for (int q = 0; q < 27; ++q)
                        if (in & (1u << OPP[q])) out |= 1u << q;
                    W.in.push_back(in);
                    W.out.push_back(out);
                }
                bool seen[256] = {false};
                for (int64_t g : W.fluid) {
                    const uint32_t tag = type[g] & 0xFFFFFu;
                    if (seen[tag]) continue;
                    seen[tag] = true;
                    const int x = (int)(g % nx), y = (int)((g / nx) % ny), z = (int)(g / ((int64_t)nx * ny));
                    neighbours(x, y, z, nb);
                    uint32_t in = (1u << 27) - 1;
                    for (int q = 0; q < 27; ++q)
                        if (nb[q] == SOLID) in &= ~(1u << OPP[q]);
                    uint32_t out = 0;
                    for (int q = 0; q < 27; ++q)
                        if (in & (1u << OPP[q])) out |= 1u << q;
                    tag_in[tag] = in;
                    tag_out[tag] = out;
                }
            }
        }
        // reference blocks that are never updated: active mask read at by * GX + bx
        const int GX = nx / 8, GY = ny / 8;
        std::vector<char> act((size_t)GX * GY, 0);
        for (int by = 0; by < GY; ++by)
            for (int bx = 0; bx < GX; ++bx) {
                bool any = false;
                for (int z = 0; z < 4; ++z)
                    for (int y = by * 8; y < by * 8 + 8; ++y)
                        for (int x = bx * 8; x < bx * 8 + 8; ++x) any = any || cls(idx(x, y, z)) != SOLID;
                act[(size_t)by * GX + bx] = any;
            }
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x) frozen[idx(x, y, z)] = !act[(size_t)(y / 8) * GX + x / 8];
        return "";
    }

    // ---------------- closures ------------------------------------------------------------
    // update_neumaan_density_velocity (boundaries.cuh:163-199): pre-stream x-1 neighbour,
    // blended with the node itself by |u_x| when the outlet is convective.
    // With NEUMANN_CURRENT_UPDATE (current_update_neumaan_density_velocity, boundaries.cuh:96-161)
    // both are the post-stream sums instead: of the x-1 neighbour's streamed populations and
    // of the node's own `p`, accumulated in q order.
    M10<T> streamed_rho_u(const T *f) const {
        M10<T> m{};
        T r = 0, jx = 0, jy = 0, jz = 0;
        for (int q = 0; q < 27; ++q) {
            r += f[q];
            jx += f[q] * (T)CX[q];
            jy += f[q] * (T)CY[q];
            jz += f[q] * (T)CZ[q];
        }
        const T inv = (T)1 / r;
        m.rho = r;
        m.ux = jx * inv;
        m.uy = jy * inv;
        m.uz = jz * inv;
        return m;
    }

    void neumann(int64_t i, const T *p, T &rho, T &ux, T &uy, T &uz) const {
        M10<T> a = load(i - 1);
        M10<T> b = load(i);
        if (d.neumann_current_update) {
            const int x = (int)((i - 1) % nx), y = (int)(((i - 1) / nx) % ny), z = (int)((i - 1) / ((int64_t)nx * ny));
            T f[27];
            for (int q = 0; q < 27; ++q) {
                const int xs = (x - CX[q] + nx) % nx, ys = (y - CY[q] + ny) % ny, zs = (z - CZ[q] + nz) % nz;
                f[q] = pops[27 * idx(xs, ys, zs) + q];
            }
            a = streamed_rho_u(f);
            b = streamed_rho_u(p);
        }
        if (d.convective_outlet) {
            const T uc = std::sqrt(a.ux * a.ux);
            rho = (T)((1.0 - (double)uc) * (double)b.rho + (double)(uc * a.rho));
            ux = (T)((1.0 - (double)uc) * (double)b.ux + (double)(uc * a.ux));
            uy = (T)((1.0 - (double)uc) * (double)b.uy + (double)(uc * a.uy));
            uz = (T)((1.0 - (double)uc) * (double)b.uz + (double)(uc * a.uz));
        } else {
            rho = a.rho; ux = a.ux; uy = a.uy; uz = a.uz;
        }
    }

    // boundary_condition (boundaries.cuh:201-843).  f: streamed populations, m: pre-stream.
    void planar(uint32_t c, int64_t i, const T *p, M10<T> &m) const {
        const T one = 1, O = omega;
        T &rho = m.rho, &ux = m.ux, &uy = m.uy, &uz = m.uz;
        T &mxx = m.mxx, &myy = m.myy, &mzz = m.mzz, &mxy = m.mxy, &mxz = m.mxz, &myz = m.myz;
        auto zero_m = [&]() { mxx = myy = mzz = mxy = mxz = myz = 0; };
        switch (c) {
            case WEST: {
                const T rI = p[0] + p[2] + p[3] + p[4] + p[5] + p[6] + p[8] + p[10] + p[11] + p[12] + p[14] + p[16] + p[17] +
                             p[18] + p[20] + p[22] + p[24] + p[25];
                const T iv = one / rI;
                const T mxyI = ((p[8] + p[20] + p[22]) - (p[14] + p[24] + p[25])) * iv;
                const T mxzI = ((p[10] + p[20] + p[24]) - (p[16] + p[22] + p[25])) * iv;
                rho = -(T)6 * rI / (-(T)5 + (T)3 * ux + (T)3 * ux * ux);
                ux = umax; uy = 0; uz = 0;
                mxx = ux * ux; myy = 0; mzz = 0;
                mxy = (T)2 * mxyI * rI / rho;
                mxz = (T)2 * mxzI * rI / rho;
                myz = 0;
                return;
            }
            case EAST: {
                const T rI = p[0] + p[1] + p[3] + p[4] + p[5] + p[6] + p[7] + p[9] + p[11] + p[12] + p[13] + p[15] + p[17] +
                             p[18] + p[19] + p[21] + p[23] + p[26];
                const T iv = one / rI;
                const T myyI = (p[3] + p[4] + p[7] + p[11] + p[12] + p[13] + p[17] + p[18] + p[19] + p[21] + p[23] + p[26]) * iv - L.cs2;
                const T mzzI = (p[5] + p[6] + p[9] + p[11] + p[12] + p[15] + p[17] + p[18] + p[19] + p[21] + p[23] + p[26]) * iv - L.cs2;
                const T mxyI = ((p[7] + p[19] + p[21]) - (p[13] + p[23] + p[26])) * iv;
                const T mxzI = ((p[9] + p[19] + p[23]) - (p[15] + p[21] + p[26])) * iv;
                const T myzI = (p[11] + p[12] - p[17] - p[18] + p[19] - p[21] - p[23] + p[26]) * iv;
                neumann(i, p, rho, ux, uy, uz);
                mxx = ux * ux;
                myy = ((T)6 * myyI * rI - (T)6 * mzzI * rI + (T)5 * uy * uy * rho + (T)5 * uz * uz * rho) / ((T)10 * rho);
                mzz = (-(T)6 * myyI * rI + (T)6 * mzzI * rI + (T)5 * uy * uy * rho + (T)5 * uz * uz * rho) / ((T)10 * rho);
                mxy = ((T)6 * mxyI * rI - uy * rho) / ((T)3 * rho);
                mxz = ((T)6 * mxzI * rI - uz * rho) / ((T)3 * rho);
                myz = (T)6 * myzI * rI / ((T)5 * rho);
                return;
            }
            case NORTH:
            case SOUTH: {
                const bool n = c == NORTH;
                const T rI = n ? p[0] + p[1] + p[2] + p[3] + p[5] + p[6] + p[7] + p[9] + p[10] + p[11] + p[14] + p[15] + p[16] +
                                     p[17] + p[19] + p[21] + p[24] + p[25]
                               : p[0] + p[1] + p[2] + p[4] + p[5] + p[6] + p[8] + p[9] + p[10] + p[12] + p[13] + p[15] + p[16] +
                                     p[18] + p[20] + p[22] + p[23] + p[26];
                const T iv = one / rI;
                const T mxyI = n ? ((p[7] + p[19] + p[21]) - (p[14] + p[24] + p[25])) * iv
                                 : ((p[8] + p[20] + p[22]) - (p[13] + p[23] + p[26])) * iv;
                const T myzI = n ? ((p[11] + p[19] + p[25]) - (p[17] + p[21] + p[24])) * iv
                                 : ((p[12] + p[20] + p[26]) - (p[18] + p[22] + p[23])) * iv;
                rho = (T)6 * rI / (T)5;
                ux = uy = uz = 0;
                zero_m();
                mxy = (T)2 * mxyI * rI / rho;
                myz = (T)2 * myzI * rI / rho;
                return;
            }
            case BACK:
            case FRONT: {
                const bool f = c == FRONT;
                const T rI = f ? p[0] + p[1] + p[2] + p[3] + p[4] + p[5] + p[7] + p[8] + p[9] + p[11] + p[13] + p[14] + p[16] +
                                     p[18] + p[19] + p[22] + p[23] + p[25]
                               : p[0] + p[1] + p[2] + p[3] + p[4] + p[6] + p[7] + p[8] + p[10] + p[12] + p[13] + p[14] + p[15] +
                                     p[17] + p[20] + p[21] + p[24] + p[26];
                const T iv = one / rI;
                const T mxzI = f ? ((p[9] + p[19] + p[23]) - (p[16] + p[22] + p[25])) * iv
                                 : ((p[10] + p[20] + p[24]) - (p[15] + p[21] + p[26])) * iv;
                const T myzI = f ? ((p[11] + p[19] + p[25]) - (p[18] + p[22] + p[23])) * iv
                                 : ((p[12] + p[20] + p[26]) - (p[17] + p[21] + p[24])) * iv;
                rho = (T)6 * rI / (T)5;
                ux = uy = uz = 0;
                zero_m();
                mxz = (T)2 * mxzI * rI / rho;
                myz = (T)2 * myzI * rI / rho;
                return;
            }
            default: break;
        }
        // edges: table of (known-population sum, the normal-pair moment, the side moment)
        // Per edge: the 12 known populations, the normal-pair moment as +(3 pops) or -(3 pops),
        // the x-edge side moment m_yz as a signed 4-term sum (left to right), which moment the
        // pair is, and the sign s of (36 m_I rho_I + s rho).
        struct Edge {
            uint32_t c;
            int rq[12];
            int pos[3], neg[3];
            int sq[4], ss[4];
            int side;
            int pair;  // 0: mxy, 1: mxz, 2: myz
            int sign;
            bool east;
        };
        static const Edge E[] = {
            {NORTH_WEST, {0, 2, 3, 5, 6, 10, 11, 14, 16, 17, 24, 25}, {-1, -1, -1}, {14, 24, 25}, {11, 17, 24, 25}, {1, -1, -1, 1}, 1, 0, 1, false},
            {SOUTH_WEST, {0, 2, 4, 5, 6, 8, 10, 12, 16, 18, 20, 22}, {8, 20, 22}, {-1, -1, -1}, {12, 18, 20, 22}, {1, -1, 1, -1}, 1, 0, -1, false},
            {WEST_FRONT, {0, 2, 3, 4, 5, 8, 11, 14, 16, 18, 22, 25}, {-1, -1, -1}, {16, 22, 25}, {11, 18, 22, 25}, {1, -1, -1, 1}, 1, 1, 1, false},
            {WEST_BACK, {0, 2, 3, 4, 6, 8, 10, 12, 14, 17, 20, 24}, {10, 20, 24}, {-1, -1, -1}, {12, 17, 20, 24}, {1, -1, 1, -1}, 1, 1, -1, false},
            {NORTH_EAST, {0, 1, 3, 5, 6, 7, 9, 11, 15, 17, 19, 21}, {7, 19, 21}, {-1, -1, -1}, {11, 17, 19, 21}, {1, -1, 1, -1}, 1, 0, -1, true},
            {SOUTH_EAST, {0, 1, 4, 5, 6, 9, 12, 13, 15, 18, 23, 26}, {-1, -1, -1}, {13, 23, 26}, {12, 18, 23, 26}, {1, -1, -1, 1}, 1, 0, 1, true},
            {EAST_FRONT, {0, 1, 3, 4, 5, 7, 9, 11, 13, 18, 19, 23}, {9, 19, 23}, {-1, -1, -1}, {11, 18, 19, 23}, {1, -1, 1, -1}, 1, 1, -1, true},
            {EAST_BACK, {0, 1, 3, 4, 6, 7, 12, 13, 15, 17, 21, 26}, {-1, -1, -1}, {15, 21, 26}, {12, 17, 21, 26}, {1, -1, -1, 1}, 1, 1, 1, true},
            {NORTH_FRONT, {0, 1, 2, 3, 5, 7, 9, 11, 14, 16, 19, 25}, {11, 19, 25}, {-1, -1, -1}, {0, 0, 0, 0}, {0, 0, 0, 0}, 0, 2, -1, false},
            {NORTH_BACK, {0, 1, 2, 3, 6, 7, 10, 14, 15, 17, 21, 24}, {-1, -1, -1}, {17, 21, 24}, {0, 0, 0, 0}, {0, 0, 0, 0}, 0, 2, 1, false},
            {SOUTH_FRONT, {0, 1, 2, 4, 5, 8, 9, 13, 16, 18, 22, 23}, {-1, -1, -1}, {18, 22, 23}, {0, 0, 0, 0}, {0, 0, 0, 0}, 0, 2, 1, false},
            {SOUTH_BACK, {0, 1, 2, 4, 6, 8, 10, 12, 13, 15, 20, 26}, {12, 20, 26}, {-1, -1, -1}, {0, 0, 0, 0}, {0, 0, 0, 0}, 0, 2, -1, false},
        };
        for (const Edge &e : E) {
            if (e.c != c) continue;
            T rI = 0;
            for (int k = 0; k < 12; ++k) rI += p[e.rq[k]];
            const T iv = one / rI;
            T s = 0;
            if (e.pos[0] >= 0) s = (p[e.pos[0]] + p[e.pos[1]] + p[e.pos[2]]);
            else s = -(p[e.neg[0]] + p[e.neg[1]] + p[e.neg[2]]);
            const T mI = s * iv;
            T side = p[e.sq[0]];
            for (int k = 1; k < 4; ++k) side = e.ss[k] > 0 ? side + p[e.sq[k]] : side - p[e.sq[k]];
            const T sideI = e.side ? side * iv : (T)0;
            if (e.east) {
                neumann(i, p, rho, ux, uy, uz);
            } else {
                rho = e.sign > 0 ? (T)36 * rI * (one + mI - mI * O) / ((T)24 + O)
                                 : (T)36 * rI * (one - mI + mI * O) / ((T)24 + O);
                ux = uy = uz = 0;
            }
            zero_m();
            const T pair = e.sign > 0 ? ((T)36 * mI * rI + rho) / ((T)9 * rho) : ((T)36 * mI * rI - rho) / ((T)9 * rho);
            if (e.pair == 0) mxy = pair;
            else if (e.pair == 1) mxz = pair;
            else myz = pair;
            if (e.side) myz = (T)12 * sideI * rI / ((T)5 * rho);
            return;
        }
        // corners
        static const struct { uint32_t c; int rq[8]; bool east; } K[] = {
            {NWF, {0, 2, 3, 5, 11, 14, 16, 25}, false}, {NWB, {0, 2, 3, 6, 10, 14, 17, 24}, false},
            {SWF, {0, 2, 4, 5, 8, 16, 18, 22}, false},  {SWB, {0, 2, 4, 6, 8, 10, 12, 20}, false},
            {NEF, {0}, true}, {NEB, {0}, true}, {SEF, {0}, true}, {SEB, {0}, true}};
        for (const auto &k : K) {
            if (k.c != c) continue;
            if (k.east) {
                neumann(i, p, rho, ux, uy, uz);
            } else {
                T rI = 0;
                for (int j = 0; j < 8; ++j) rI += p[k.rq[j]];
                rho = (T)216 * rI / (T)125;
                ux = uy = uz = 0;
            }
            zero_m();
            return;
        }
    }

    // fluid_boundary_condition (boundaries.cuh:845-1037), Equilibrium and Strong rules
    void bcfluid(uint32_t tag, const T *p, M10<T> &m) const {
        T rI = 0, uxI = 0, uyI = 0, uzI = 0, mxxI = 0, myyI = 0, mzzI = 0, mxyI = 0, mxzI = 0, myzI = 0;
        const uint32_t mask = tag_in[tag];
        for (int q = 0; q < 27; ++q) {
            if (!(mask & (1u << q))) continue;
            const T f = p[q];
            rI += f;
            uxI += f * (T)CX[q]; uyI += f * (T)CY[q]; uzI += f * (T)CZ[q];
            mxxI += f * L.hxx[q]; myyI += f * L.hyy[q]; mzzI += f * L.hzz[q];
            mxyI += f * L.hxy[q]; mxzI += f * L.hxz[q]; myzI += f * L.hyz[q];
        }
        const T iv = (T)1 / rI;
        uxI *= iv; uyI *= iv; uzI *= iv; mxxI *= iv; myyI *= iv; mzzI *= iv; mxyI *= iv; mxzI *= iv; myzI *= iv;
        const T O = omega;
        T a, b, c;
        auto pick = [&](T a_, T b_, T c_) {
            const T disc = std::max(b_ * b_ - (T)4 * a_ * c_, (T)0);
            const T r1 = (-b_ + std::sqrt(disc)) / ((T)2 * a_);
            const T r2 = (-b_ - std::sqrt(disc)) / ((T)2 * a_);
            return (r1 > 0 && std::fabs(r1 - rI) < std::fabs(r2 - rI)) ? r1 : r2;
        };
        T &rho = m.rho;
        const bool strong = d.bcf_mass_bc == MRLBM_MASS_STRONG;
        switch (tag) {
            case 17: {
                const T cpoly = (T)45 * (mxxI * mxxI) + (T)405 * (mxyI * mxyI) + (T)45 * (myyI * myyI) + (T)345 * myyI * uxI +
                                (T)589 * (uxI * uxI) + (T)345 * myyI * uyI + (T)1467 * uxI * uyI + (T)589 * (uyI * uyI) +
                                (T)45 * mxyI * ((T)6 * myyI + (T)23 * (uxI + uyI)) +
                                (T)15 * mxxI * ((T)18 * mxyI + (T)6 * myyI + (T)23 * (uxI + uyI));
                if (strong) {
                    a = (T)-9996 - (T)206 * O;
                    b = (T)-6 * rI * ((T)12 * mxxI * ((T)-17 + (T)20 * O) -
                                      (T)17 * ((T)102 + (T)36 * mxyI + (T)12 * myyI - (T)5 * uxI - (T)5 * uyI) +
                                      O * ((T)720 * mxyI + (T)240 * myyI + (T)53 * (uxI + uyI)));
                    c = (T)3 * O * (rI * rI) * cpoly;
                } else {
                    a = (T)-9998;
                    b = (T)6 * rI * ((T)1734 + (T)66 * mxxI + (T)198 * mxyI + (T)66 * myyI + (T)253 * uxI + (T)253 * uyI);
                    c = (T)3 * (rI * rI) * cpoly;
                }
                rho = pick(a, b, c);
                m.ux = ((T)3 * mxxI * rI + (T)9 * mxyI * rI + (T)3 * myyI * rI + (T)20 * rI * uxI + (T)3 * rI * uyI + rho) / ((T)17 * rho);
                m.uy = ((T)3 * mxxI * rI + (T)9 * mxyI * rI + (T)3 * myyI * rI + (T)3 * rI * uxI + (T)20 * rI * uyI + rho) / ((T)17 * rho);
                m.uz = ((T)3 * rI * (mxzI + myzI + (T)10 * uzI)) / ((T)29 * rho);
                m.mxx = ((T)57 * mxxI * rI + (T)18 * mxyI * rI + (T)6 * myyI * rI + (T)6 * rI * uxI + (T)6 * rI * uyI + (T)2 * rho) / ((T)51 * rho);
                m.myy = ((T)6 * mxxI * rI + (T)18 * mxyI * rI + (T)57 * myyI * rI + (T)6 * rI * uxI + (T)6 * rI * uyI + (T)2 * rho) / ((T)51 * rho);
                m.mzz = ((T)36 * mzzI * rI) / ((T)35 * rho);
                m.mxy = ((T)3 * mxxI * rI + (T)26 * mxyI * rI + (T)3 * myyI * rI + (T)3 * rI * uxI + (T)3 * rI * uyI + rho) / ((T)17 * rho);
                m.mxz = (rI * ((T)32 * mxzI + (T)3 * myzI + uzI)) / ((T)29 * rho);
                m.myz = (rI * ((T)3 * mxzI + (T)32 * myzI + uzI)) / ((T)29 * rho);
                return;
            }
            case 34: {
                const T cpoly = (T)45 * (mxxI * mxxI) + (T)405 * (mxyI * mxyI) + (T)45 * (myyI * myyI) - (T)345 * myyI * uxI +
                                (T)589 * (uxI * uxI) + (T)345 * myyI * uyI - (T)1467 * uxI * uyI + (T)589 * (uyI * uyI) -
                                (T)45 * mxyI * ((T)6 * myyI - (T)23 * uxI + (T)23 * uyI) +
                                (T)15 * mxxI * ((T)-18 * mxyI + (T)6 * myyI - (T)23 * uxI + (T)23 * uyI);
                if (strong) {
                    a = (T)9996 + (T)206 * O;
                    b = (T)6 * rI * (mxyI * ((T)612 - (T)720 * O) + (T)240 * myyI * O + (T)12 * mxxI * ((T)-17 + (T)20 * O) -
                                     (T)17 * ((T)102 + (T)12 * myyI + (T)5 * uxI - (T)5 * uyI) + (T)53 * O * (-uxI + uyI));
                    c = (T)-3 * O * (rI * rI) * cpoly;
                } else {
                    a = (T)-9998;
                    b = (T)6 * rI * ((T)1734 + (T)66 * mxxI - (T)198 * mxyI + (T)66 * myyI - (T)253 * uxI + (T)253 * uyI);
                    c = (T)3 * (rI * rI) * cpoly;
                }
                rho = pick(a, b, c);
                m.ux = -((T)3 * mxxI * rI - (T)9 * mxyI * rI + (T)3 * myyI * rI - (T)20 * rI * uxI + (T)3 * rI * uyI + rho) / ((T)17 * rho);
                m.uy = ((T)3 * mxxI * rI - (T)9 * mxyI * rI + (T)3 * myyI * rI - (T)3 * rI * uxI + (T)20 * rI * uyI + rho) / ((T)17 * rho);
                m.uz = ((T)3 * rI * (-mxzI + myzI + (T)10 * uzI)) / ((T)29 * rho);
                m.mxx = ((T)57 * mxxI * rI - (T)18 * mxyI * rI + (T)6 * myyI * rI - (T)6 * rI * uxI + (T)6 * rI * uyI + (T)2 * rho) / ((T)51 * rho);
                m.myy = ((T)6 * mxxI * rI - (T)18 * mxyI * rI + (T)57 * myyI * rI - (T)6 * rI * uxI + (T)6 * rI * uyI + (T)2 * rho) / ((T)51 * rho);
                m.mzz = ((T)36 * mzzI * rI) / ((T)35 * rho);
                m.mxy = -((T)3 * mxxI * rI - (T)26 * mxyI * rI + (T)3 * myyI * rI - (T)3 * rI * uxI + (T)3 * rI * uyI + rho) / ((T)17 * rho);
                m.mxz = (rI * ((T)32 * mxzI - (T)3 * myzI - uzI)) / ((T)29 * rho);
                m.myz = (rI * ((T)-3 * mxzI + (T)32 * myzI + uzI)) / ((T)29 * rho);
                return;
            }
            case 68: {
                const T cpoly = (T)45 * (mxxI * mxxI) + (T)405 * (mxyI * mxyI) + (T)45 * (myyI * myyI) + (T)345 * myyI * uxI +
                                (T)589 * (uxI * uxI) - (T)45 * mxyI * ((T)6 * myyI + (T)23 * uxI - (T)23 * uyI) +
                                (T)15 * mxxI * ((T)-18 * mxyI + (T)6 * myyI + (T)23 * uxI - (T)23 * uyI) - (T)345 * myyI * uyI -
                                (T)1467 * uxI * uyI + (T)589 * (uyI * uyI);
                if (strong) {
                    a = (T)9996 + (T)206 * O;
                    b = (T)6 * rI * (mxyI * ((T)612 - (T)720 * O) + (T)240 * myyI * O + (T)12 * mxxI * ((T)-17 + (T)20 * O) +
                                     (T)53 * O * (uxI - uyI) - (T)17 * ((T)102 + (T)12 * myyI - (T)5 * uxI + (T)5 * uyI));
                    c = (T)-3 * O * (rI * rI) * cpoly;
                } else {
                    a = (T)-9998;
                    b = (T)6 * rI * ((T)1734 + (T)66 * mxxI - (T)198 * mxyI + (T)66 * myyI + (T)253 * uxI - (T)253 * uyI);
                    c = (T)3 * (rI * rI) * cpoly;
                }
                rho = pick(a, b, c);
                m.ux = ((T)3 * mxxI * rI - (T)9 * mxyI * rI + (T)3 * myyI * rI + (T)20 * rI * uxI - (T)3 * rI * uyI + rho) / ((T)17 * rho);
                m.uy = -((T)3 * mxxI * rI - (T)9 * mxyI * rI + (T)3 * myyI * rI + (T)3 * rI * uxI - (T)20 * rI * uyI + rho) / ((T)17 * rho);
                m.uz = ((T)3 * rI * (mxzI - myzI + (T)10 * uzI)) / ((T)29 * rho);
                m.mxx = ((T)57 * mxxI * rI - (T)18 * mxyI * rI + (T)6 * myyI * rI + (T)6 * rI * uxI - (T)6 * rI * uyI + (T)2 * rho) / ((T)51 * rho);
                m.myy = ((T)6 * mxxI * rI - (T)18 * mxyI * rI + (T)57 * myyI * rI + (T)6 * rI * uxI - (T)6 * rI * uyI + (T)2 * rho) / ((T)51 * rho);
                m.mzz = ((T)36 * mzzI * rI) / ((T)35 * rho);
                m.mxy = -((T)3 * mxxI * rI - (T)26 * mxyI * rI + (T)3 * myyI * rI + (T)3 * rI * uxI - (T)3 * rI * uyI + rho) / ((T)17 * rho);
                m.mxz = (rI * ((T)32 * mxzI - (T)3 * myzI + uzI)) / ((T)29 * rho);
                m.myz = -(rI * ((T)3 * mxzI - (T)32 * myzI + uzI)) / ((T)29 * rho);
                return;
            }
            case 136: {
                const T cpoly = (T)45 * (mxxI * mxxI) + (T)405 * (mxyI * mxyI) + (T)45 * (myyI * myyI) - (T)345 * myyI * uxI +
                                (T)589 * (uxI * uxI) - (T)345 * myyI * uyI + (T)1467 * uxI * uyI + (T)589 * (uyI * uyI) +
                                (T)45 * mxyI * ((T)6 * myyI - (T)23 * (uxI + uyI)) +
                                (T)15 * mxxI * ((T)18 * mxyI + (T)6 * myyI - (T)23 * (uxI + uyI));
                if (strong) {
                    a = (T)-9996 - (T)206 * O;
                    b = (T)-6 * rI * ((T)12 * mxxI * ((T)-17 + (T)20 * O) -
                                      (T)17 * ((T)102 + (T)36 * mxyI + (T)12 * myyI + (T)5 * uxI + (T)5 * uyI) +
                                      O * ((T)720 * mxyI + (T)240 * myyI - (T)53 * (uxI + uyI)));
                    c = (T)3 * O * (rI * rI) * cpoly;
                } else {
                    a = (T)-9998;
                    b = (T)6 * rI * ((T)1734 + (T)66 * mxxI + (T)198 * mxyI + (T)66 * myyI - (T)253 * uxI - (T)253 * uyI);
                    c = (T)3 * (rI * rI) * cpoly;
                }
                rho = pick(a, b, c);
                m.ux = -((T)3 * mxxI * rI + (T)9 * mxyI * rI + (T)3 * myyI * rI - (T)20 * rI * uxI - (T)3 * rI * uyI + rho) / ((T)17 * rho);
                m.uy = -((T)3 * mxxI * rI + (T)9 * mxyI * rI + (T)3 * myyI * rI - (T)3 * rI * uxI - (T)20 * rI * uyI + rho) / ((T)17 * rho);
                m.uz = ((T)-3 * rI * (mxzI + myzI - (T)10 * uzI)) / ((T)29 * rho);
                m.mxx = ((T)57 * mxxI * rI + (T)18 * mxyI * rI + (T)6 * myyI * rI - (T)6 * rI * uxI - (T)6 * rI * uyI + (T)2 * rho) / ((T)51 * rho);
                m.myy = ((T)6 * mxxI * rI + (T)18 * mxyI * rI + (T)57 * myyI * rI - (T)6 * rI * uxI - (T)6 * rI * uyI + (T)2 * rho) / ((T)51 * rho);
                m.mzz = ((T)36 * mzzI * rI) / ((T)35 * rho);
                m.mxy = ((T)3 * mxxI * rI + (T)26 * mxyI * rI + (T)3 * myyI * rI - (T)3 * rI * uxI - (T)3 * rI * uyI + rho) / ((T)17 * rho);
                m.mxz = (rI * ((T)32 * mxzI + (T)3 * myzI - uzI)) / ((T)29 * rho);
                m.myz = (rI * ((T)3 * mxzI + (T)32 * myzI - uzI)) / ((T)29 * rho);
                return;
            }
            default: return;  // other tags keep the pre-stream moments
        }
    }

    // bcsolid_boundary_condition (boundaries.cuh:1039-1214), z walls only.  Per tag: the 16
    // populations the reference sums into rhoI, and the signs (px, py) with which its incoming
    // mxzI, myzI enter rho, mxz and myz (TAG_BCS_1..8 = 7, 11, 13, 14, 112, 176, 208, 224).
    void bcsolid(uint32_t tag, const T *p, M10<T> &m) const {
        struct Row { uint32_t tag; int known[16]; int px, py; };
        static const Row rows[8] = {
            {7, {0, 1, 2, 3, 4, 5, 7, 9, 11, 13, 14, 16, 18, 19, 23, 25}, -1, -1},
            {11, {0, 1, 2, 3, 4, 5, 7, 8, 9, 11, 14, 16, 18, 19, 22, 25}, 1, -1},
            {13, {0, 1, 2, 3, 4, 5, 7, 8, 9, 11, 13, 16, 18, 19, 22, 23}, -1, 1},
            {14, {0, 1, 2, 3, 4, 5, 8, 9, 11, 13, 14, 16, 18, 22, 23, 25}, 1, 1},
            {112, {0, 1, 2, 3, 4, 6, 7, 10, 12, 13, 14, 15, 17, 21, 24, 26}, 1, 1},
            {176, {0, 1, 2, 3, 4, 6, 7, 8, 10, 12, 14, 15, 17, 20, 21, 24}, -1, 1},
            {208, {0, 1, 2, 3, 4, 6, 7, 8, 10, 12, 13, 15, 17, 20, 21, 26}, 1, -1},
            {224, {0, 1, 2, 3, 4, 6, 8, 10, 12, 13, 14, 15, 17, 20, 24, 26}, -1, -1},
        };
        const Row *row = nullptr;
        for (const Row &r : rows)
            if (r.tag == tag) row = &r;
        if (!row) return;  // other tags keep the pre-stream moments
        T rI = 0, sxz = 0, syz = 0;
        for (int k = 0; k < 16; ++k) {
            const int q = row->known[k];
            rI += p[q];
            const int xz = CX[q] * CZ[q], yz = CY[q] * CZ[q];
            if (xz > 0) sxz += p[q]; else if (xz < 0) sxz -= p[q];
            if (yz > 0) syz += p[q]; else if (yz < 0) syz -= p[q];
        }
        const T iv = (T)(1.0 / (double)rI);
        const T mxzI = sxz * iv, myzI = syz * iv;
        const T px = (T)row->px, py = (T)row->py, O = omega;
        const T rho = ((T)108 * ((T)10 - (O - (T)1) * (px * mxzI) - (O - (T)1) * (py * myzI)) * rI) / ((T)874 + O);
        m.rho = rho;
        m.ux = m.uy = m.uz = 0;
        m.mxx = m.myy = m.mzz = m.mxy = 0;
        m.mxz = ((T)198 * mxzI * rI + (T)18 * (px * py) * myzI * rI + px * rho) / ((T)90 * rho);
        m.myz = ((T)18 * (px * py) * mxzI * rI + (T)198 * myzI * rI + py * rho) / ((T)90 * rho);
    }

    // evaluate_incoming_moments_rotated (curvedLBM.cu:5-59)
    void incoming_rot(T c, T s, uint32_t mask, const T *p, M10<T> &m) const {
        T r = 0, a = 0, b = 0, e = 0, f = 0, g = 0, h = 0;
        for (int q = 0; q < 27; ++q) {
            if (!(mask & (1u << q))) continue;
            const T cx = (T)CX[q], cy = (T)CY[q], cz = (T)CZ[q];
            const T xp = cx * c + cy * s, yp = -cx * s + cy * c, zp = cz;
            r += p[q];
            a += p[q] * (xp * xp - L.cs2);
            b += p[q] * (yp * yp - L.cs2);
            e += p[q] * (zp * zp - L.cs2);
            f += p[q] * (xp * yp);
            g += p[q] * (xp * zp);
            h += p[q] * (yp * zp);
        }
        const T iv = (T)1 / r;
        m.rho = r;
        m.mxx = a * iv; m.myy = b * iv; m.mzz = e * iv; m.mxy = f * iv; m.mxz = g * iv; m.myz = h * iv;
    }

    T bilinear(const std::vector<T> &arr, T x, T y, int z) const {
        const int x0 = (int)std::floor(x), y0 = (int)std::floor(y);
        const T xd = x - (T)x0, yd = y - (T)y0;
        const T q00 = arr[idx(x0, y0, z)], q10 = arr[idx(x0 + 1, y0, z)];
        const T q01 = arr[idx(x0, y0 + 1, z)], q11 = arr[idx(x0 + 1, y0 + 1, z)];
        const T r0 = ((T)1 - xd) * q00 + xd * q10;
        const T r1 = ((T)1 - xd) * q01 + xd * q11;
        return ((T)1 - yd) * r0 + yd * r1;
    }

    // curved_boundary_condition_rotated and the numerical solutions (curvedLBM.cu:61-132,
    // numerical_solution.cu:4-279); `snap` are the post-stream moment arrays.
    void curved(int w, size_t bi, const std::vector<T> *snap, M10<T> &m) const {
        const WallO &W = wall[w];
        const int64_t g = W.list[bi];
        const int x = (int)(g % nx), y = (int)((g / nx) % ny), z = (int)(g / ((int64_t)nx * ny));
        (void)x; (void)y;
        const T c = W.nx[bi], s = W.ny[bi], delta = W.delta[bi];
        const T rwall = (T)(0.5f * d.d_wall[w]);
        const T xw = (T)d.xc + rwall * c, yw = (T)d.yc + rwall * s;
        const T dir = w == 1 ? (T)-1 : (T)1;
        const T x1 = xw + dir * c, y1 = yw + dir * s;
        const T x2 = xw + dir * (T)2 * c, y2 = yw + dir * (T)2 * s;
        T v[2][9];
        const T px[2] = {x1, x2}, py[2] = {y1, y2};
        for (int k = 0; k < 2; ++k) {
            const T ux = bilinear(snap[1], px[k], py[k], z), uy = bilinear(snap[2], px[k], py[k], z);
            const T uz = bilinear(snap[3], px[k], py[k], z);
            const T mxx = bilinear(snap[4], px[k], py[k], z), myy = bilinear(snap[5], px[k], py[k], z);
            const T mzz = bilinear(snap[6], px[k], py[k], z), mxy = bilinear(snap[7], px[k], py[k], z);
            const T mxz = bilinear(snap[8], px[k], py[k], z), myz = bilinear(snap[9], px[k], py[k], z);
            const T s2 = (T)2 * s * c, c2 = c * c - s * s;
            v[k][0] = ux * c + uy * s;
            v[k][1] = -ux * s + uy * c;
            v[k][2] = uz;
            v[k][3] = mxx * c * c + myy * s * s + mxy * s2;
            v[k][4] = mxx * s * s + myy * c * c - mxy * s2;
            v[k][5] = mzz;
            v[k][6] = mxy * c2 + (T)0.5f * (myy - mxx) * s2;
            v[k][7] = mxz * c + myz * s;
            v[k][8] = myz * c - mxz * s;
        }
        const T Uw[3] = {(T)d.wall_u[w][0], (T)d.wall_u[w][1], (T)d.wall_u[w][2]};
        auto ext = [&](T vw, T f1, T f2) {
            const T dd = delta / (T)1.0f, d2 = dd * dd;
            const T c1 = (T)1 - (T)0.5f * d2 + (T)1.5f * dd, c2 = d2 - (T)2 * dd, c3 = -(T)0.5f * (d2 - dd);
            return c1 * vw + c2 * f1 + c3 * f2;
        };
        const T uxp = ext(Uw[0], v[0][0], v[1][0]), uyp = ext(Uw[1], v[0][1], v[1][1]), uzp = ext(Uw[2], v[0][2], v[1][2]);
        const T mxxp = ext(Uw[0] * Uw[0], v[0][3], v[1][3]), myyp = ext(Uw[1] * Uw[1], v[0][4], v[1][4]);
        const T mzzp = ext(Uw[2] * Uw[2], v[0][5], v[1][5]), myzp = ext(Uw[1] * Uw[2], v[0][8], v[1][8]);
        const uint32_t in = W.in[bi], out = W.out[bi];
        const bool strong = d.mass_bc == MRLBM_MASS_STRONG;
        const T s2 = (T)2 * s * c, c2 = c * c - s * s;
        const T cbf = (T)0.5f * L.as2 * L.as2;
        T A = 0, E = 0, B[6] = {0, 0, 0, 0, 0, 0}, Dxy = 0, Dxz = 0, Fy[6] = {0, 0, 0, 0, 0, 0}, Fz[6] = {0, 0, 0, 0, 0, 0};
        for (int q = 0; q < 27; ++q) {
            const T cx = (T)CX[q], cy = (T)CY[q], cz = (T)CZ[q];
            const T xp = cx * c + cy * s, yp = -cx * s + cy * c, zp = cz;
            const T H[6] = {xp * xp - L.cs2, yp * yp - L.cs2, zp * zp - L.cs2, xp * yp, xp * zp, yp * zp};
            const T wq = L.w[q], cf = cbf * wq;
            const T Ai = wq * ((T)1 + L.as2 * (uxp * xp + uyp * yp + uzp * zp));
            const T Ei = Ai + cf * (uxp * uxp * H[0] + uyp * uyp * H[1] + uzp * uzp * H[2] + (T)2 * uxp * uyp * H[3] +
                                    (T)2 * uxp * uzp * H[4] + (T)2 * uyp * uzp * H[5]);
            if (strong && (out & (1u << q))) {
                A += Ai;
                E += Ei;
                for (int k = 0; k < 6; ++k) B[k] += cf * H[k];
            }
            if (in & (1u << q)) {
                if (!strong) E += Ei;
                Dxy += Ai * H[3];
                Dxz += Ai * H[4];
                for (int k = 0; k < 6; ++k) {
                    Fy[k] += (cf * H[k]) * H[3];
                    Fz[k] += (cf * H[k]) * H[4];
                }
            }
        }
        const T rIp = m.rho, mxyIp = m.mxy, mxzIp = m.mxz;
        T G = E;
        if (strong) {
            const T om = (T)1 - omega;
            G = om * A + omega * E;
            for (int k = 0; k < 6; ++k) {
                Fy[k] -= (om * mxyIp) * B[k];
                Fz[k] -= (om * mxzIp) * B[k];
            }
        }
        const T Rxy = G * mxyIp - Dxy, Rxz = G * mxzIp - Dxz;
        const T a1 = (T)2 * Fy[3], b1 = (T)2 * Fy[4];
        const T c1 = Rxy - mxxp * Fy[0] - myyp * Fy[1] - mzzp * Fy[2] - (T)2 * myzp * Fy[5];
        const T a2 = (T)2 * Fz[3], b2 = (T)2 * Fz[4];
        const T cc2 = Rxz - mxxp * Fz[0] - myyp * Fz[1] - mzzp * Fz[2] - (T)2 * myzp * Fz[5];
        const T inv = (T)1 / (a2 * b1 - a1 * b2);
        const T mxyp = (b1 * cc2 - b2 * c1) * inv, mxzp = (a2 * c1 - a1 * cc2) * inv;
        m.ux = uxp * c - uyp * s;
        m.uy = uxp * s + uyp * c;
        m.uz = uzp;
        m.mxx = mxxp * c * c + myyp * s * s - mxyp * s2;
        m.myy = mxxp * s * s + myyp * c * c + mxyp * s2;
        m.mzz = mzzp;
        m.mxy = (mxxp - myyp) * (T)0.5f * s2 + mxyp * c2;
        m.mxz = mxzp * c - myzp * s;
        m.myz = mxzp * s + myzp * c;
        if (strong) {
            const T om = (T)1 - omega;
            m.rho = rIp / (G + om * (mxxp * B[0] + myyp * B[1] + mzzp * B[2] + (T)2 * mxyp * B[3] + (T)2 * mxzp * B[4] +
                                     (T)2 * myzp * B[5]));
        } else {
            m.rho = rIp / E;
        }
    }

    // masked momentum sum of R(m) (forces.cu:3-23)
    void momentum(const M10<T> &m, uint32_t mask, double acc[4], double sign) const {
        T p[27];
        reconstruct(L, m, p);
        T fx = 0, fy = 0, fz = 0, fm = 0;
        for (int q = 0; q < 27; ++q) {
            if (!(mask & (1u << q))) continue;
            fx += p[q] * (T)CX[q];
            fy += p[q] * (T)CY[q];
            fz += p[q] * (T)CZ[q];
            fm += p[q];
        }
        acc[0] += sign * (double)fx;
        acc[1] += sign * (double)fy;
        acc[2] += sign * (double)fz;
        acc[3] += sign * (double)fm;
    }

    // one time step (main.cu:23-31)
    void do_step(bool want_force) {
        // kernel A: pull R(M(x - c)) with a periodic wrap, evaluate or close
        const int64_t N = n;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; ++i) reconstruct(L, load(i), &pops[27 * i]);
        std::vector<T> snap[10];
        for (int k = 0; k < 10; ++k) snap[k] = mom[k];  // pre-stream, read by the outlet
        std::vector<T> post[10];
        for (int k = 0; k < 10; ++k) post[k] = mom[k];
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; ++i) {
            if (frozen[i]) continue;
            const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((int64_t)nx * ny));
            T f[27];
            for (int q = 0; q < 27; ++q) {
                const int xs = (x - CX[q] + nx) % nx, ys = (y - CY[q] + ny) % ny, zs = (z - CZ[q] + nz) % nz;
                f[q] = pops[27 * idx(xs, ys, zs) + q];
            }
            const uint32_t c = cls(i);
            M10<T> m = load(i);  // pre-stream (state of the arrays before this step)
            if (c == BULK) {
                evaluate(L, f, m);
            } else if (c == INNER || c == OUTER) {
                const int w = c == INNER ? 0 : 1;
                const uint32_t bi = type[i] & 0xFFFFFu;
                incoming_rot((T)wall[w].nx[bi], (T)wall[w].ny[bi], wall[w].in[bi], f, m);
            } else if (c == BCF_IN || c == BCF_OUT) {
                bcfluid(type[i] & 0xFFFFFu, f, m);
            } else if (c == BCS_IN || c == BCS_OUT) {
                bcsolid(type[i] & 0xFFFFFu, f, m);
            } else if (c != SOLID) {
                planar(c, i, f, m);
            }
            post[0][i] = m.rho - rho0;
            post[1][i] = m.ux; post[2][i] = m.uy; post[3][i] = m.uz;
            post[4][i] = m.mxx; post[5][i] = m.myy; post[6][i] = m.mzz;
            post[7][i] = m.mxy; post[8][i] = m.mxz; post[9][i] = m.myz;
        }
        for (int k = 0; k < 10; ++k) mom[k].swap(post[k]);
        // curved-wall closure on the post-stream snapshot
        for (int k = 0; k < 10; ++k) snap[k] = mom[k];
        for (int w = 0; w < n_walls; ++w) {
            const int nbw = (int)wall[w].list.size();
#pragma omp parallel for schedule(static)
            for (int b = 0; b < nbw; ++b) {
                const int64_t g = wall[w].list[b];
                M10<T> m;
                m.rho = rho0 + snap[0][g];
                m.ux = snap[1][g]; m.uy = snap[2][g]; m.uz = snap[3][g];
                m.mxx = snap[4][g]; m.myy = snap[5][g]; m.mzz = snap[6][g];
                m.mxy = snap[7][g]; m.mxz = snap[8][g]; m.myz = snap[9][g];
                curved(w, b, snap, m);
                store(g, m);
            }
        }
        // incoming forces, collision, outgoing forces
        std::memset(force, 0, sizeof(force));
        if (want_force) {
            for (int w = 0; w < n_walls; ++w) {
                double acc[4] = {0, 0, 0, 0};
                double tz = 0;
                auto node_force = [&](int64_t g, uint32_t in, bool after) {
                    double a4[4] = {0, 0, 0, 0};
                    momentum(load(g), in, a4, after ? -1.0 : 1.0);
                    for (int k = 0; k < 4; ++k) acc[k] += a4[k];
                    const int x = (int)(g % nx), y = (int)((g / nx) % ny);
                    tz += ((double)x - d.xc) * a4[1] - ((double)y - d.yc) * a4[0];
                };
                for (size_t b = 0; b < wall[w].list.size(); ++b) node_force(wall[w].list[b], wall[w].in[b], false);
                for (int64_t g : wall[w].fluid) node_force(g, tag_in[type[g] & 0xFF], false);
                force[w * 5 + 0] = acc[0];
                force[w * 5 + 1] = acc[1];
                force[w * 5 + 2] = acc[2];
                force[w * 5 + 3] = acc[3];
                force[w * 5 + 4] = tz;
            }
        }
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < N; ++i) {
            if (frozen[i]) continue;
            M10<T> m = load(i);
            collide(omega, m);
            store(i, m);
        }
        if (want_force) {
            for (int w = 0; w < n_walls; ++w) {
                double acc[4] = {0, 0, 0, 0};
                double tz = 0;
                auto node_force = [&](int64_t g, uint32_t out) {
                    double a4[4] = {0, 0, 0, 0};
                    momentum(load(g), out, a4, -1.0);
                    for (int k = 0; k < 4; ++k) acc[k] += a4[k];
                    const int x = (int)(g % nx), y = (int)((g / nx) % ny);
                    tz += ((double)x - d.xc) * a4[1] - ((double)y - d.yc) * a4[0];
                };
                for (size_t b = 0; b < wall[w].list.size(); ++b) node_force(wall[w].list[b], wall[w].out[b]);
                for (int64_t g : wall[w].fluid) node_force(g, tag_out[type[g] & 0xFF]);
                for (int k = 0; k < 4; ++k) force[w * 5 + k] += acc[k];
                force[w * 5 + 4] += tz;
            }
        }
        ++step;
    }

    static unsigned hash_u(unsigned s) {
        s = (s ^ 61u) ^ (s >> 16);
        s *= 9u;
        s = s ^ (s >> 4);
        s *= 0x27d4eb2du;
        s = s ^ (s >> 15);
        return s;
    }
    static float noise(unsigned s, float scale) {
        const float r = (float)(hash_u(s) & 0x7FFFFFFFu) / (float)0x7FFFFFFF;
        return scale * (2.0f * r - 1.0f);
    }

    // initialiser (initializeLBM.cu:39-121 for the reference noise)
    void init(int kind, const double *p) {
        for (int64_t i = 0; i < n; ++i) {
            const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((int64_t)nx * ny));
            M10<T> m{};
            m.rho = rho0;
            if (kind == MRLBM_INIT_REFERENCE_NOISE) {
                const int64_t gx = nx / 8, gy = ny / 8;
                const int64_t ridx = (x % 8) + 8 * ((y % 8) + 8 * (z % 4)) + 256 * ((x / 8) + gx * ((y / 8) + gy * (z / 4)));
                const float pi = 3.14159265358979323846f;
                const float sc = 1e-4f * d.u_max;
                const double sn = std::sin(2.0 * (double)pi * (double)(float)z / (double)(float)nz);
                const float uz = (float)(1e-4 * (double)d.u_max * sn + (double)noise((unsigned)(ridx + 67890), sc));
                m.uz = (T)uz;
            } else if (kind == MRLBM_INIT_TAYLOR_GREEN) {
                const double u0 = p[0], Lw = p[1];
                const double X = x / Lw, Y = y / Lw, Z = z / Lw;
                const double u = u0 * std::sin(X) * std::cos(Y) * std::cos(Z);
                const double v = -u0 * std::cos(X) * std::sin(Y) * std::cos(Z);
                const double pr = (double)d.rho0 * u0 * u0 / 16.0 * (std::cos(2 * X) + std::cos(2 * Y)) * (std::cos(2 * Z) + 2.0);
                m.rho = (T)((double)d.rho0 + 3.0 * pr);
                m.ux = (T)u; m.uy = (T)v; m.uz = 0;
                m.mxx = (T)(u * u); m.myy = (T)(v * v); m.mxy = (T)(u * v);
            } else if (kind == MRLBM_INIT_UNIFORM || kind == MRLBM_INIT_NOISY_UNIFORM) {
                double u = p[0], v = p[1], w = p[2];
                if (kind == MRLBM_INIT_NOISY_UNIFORM) {
                    const double umag = std::sqrt(u * u + v * v + w * w), amp = p[3];
                    const unsigned base = (unsigned)i * 3u + (unsigned)p[4];
                    u += umag * amp * noise(base, 1.0f);
                    v += umag * amp * noise(base + 1u, 1.0f);
                    w += umag * amp * noise(base + 2u, 1.0f);
                }
                m.ux = (T)u; m.uy = (T)v; m.uz = (T)w;
                m.mxx = (T)(u * u); m.myy = (T)(v * v); m.mzz = (T)(w * w);
                m.mxy = (T)(u * v); m.mxz = (T)(u * w); m.myz = (T)(v * w);
            }
            store(i, m);
        }
        step = 0;
    }
};

struct Any {
    int bits;
    void *o;
};

template <typename T>
Oracle<T> *as(void *p) {
    return (Oracle<T> *)((Any *)p)->o;
}

// Relaxation rate from the physical parameters, restating the reference's constexpr chains
// (float VISC, TAU = 0.5 + 3 VISC evaluated in double and stored as float, OMEGA = 1 / TAU in
// double stored as float):
//   cylinder  VISC = U_MAX * D_WALL / RE                 MRLBM_3D/src/cases/cylinder/constants.cuh:52-54
//   annulus   VISC = U_REL * GAP / RE, as2 = 3 (float)   MRLBM_3D/src/cases/annulus/constants.cuh:73-81
//   box       VISC = U_MAX * L / RE (the Taylor-Green length L = N / 2 pi)
// This is the oracle's own derivation, independent of the product's descriptor code.  A
// descriptor without a Reynolds number carries an explicit relaxation rate instead.
float reference_omega(const mrlbm_case_desc &d) {
    if (!(d.re > 0.f)) return d.omega;
    float visc;
    double tau;
    if (d.geometry == MRLBM_GEOM_ANNULUS) {
        const float r_in = 0.5f * d.d_wall[0], r_out = 0.5f * d.d_wall[1];
        const float u_rel = std::fabs(d.wall_u[0][1] - d.wall_u[1][1]);
        visc = u_rel * (r_out - r_in) / d.re;
        const float as2 = 3.0f;
        tau = 0.5 + (double)(as2 * visc);
    } else {
        const float len = d.geometry == MRLBM_GEOM_CYLINDER ? d.d_wall[0] : d.length;
        visc = d.u_max * len / d.re;
        tau = 0.5 + 3.0 * (double)visc;
    }
    const float tau_f = (float)tau;
    return (float)(1.0 / (double)tau_f);
}

template <typename T>
void *make(const mrlbm_case_desc *d) {
    auto *o = new Oracle<T>();
    o->d = *d;
    o->nx = d->nx;
    o->ny = d->ny;
    o->nz = d->nz;
    o->n = (int64_t)d->nx * d->ny * d->nz;
    o->omega = (T)reference_omega(*d);
    o->rho0 = (T)d->rho0;
    o->umax = (T)d->u_max;
    const std::string e = o->geometry();
    if (!e.empty()) {
        g_err = e;
        delete o;
        return nullptr;
    }
    for (int k = 0; k < 10; ++k) o->mom[k].assign(o->n, (T)0);
    o->pops.assign((size_t)27 * o->n, (T)0);
    return o;
}

#define DISPATCH(p, expr)                 \
    do {                                  \
        if (((Any *)(p))->bits == 32) {   \
            auto *o = as<float>(p);       \
            expr;                         \
        } else {                          \
            auto *o = as<double>(p);      \
            expr;                         \
        }                                 \
    } while (0)

}  // namespace

extern "C" {

const char *oracle_last_error(void) { return g_err.c_str(); }

float oracle_omega(const mrlbm_case_desc *d) { return d ? reference_omega(*d) : 0.f; }

// The relaxation rate comes from reference_omega (re > 0) or the descriptor's explicit omega.
// bits = 32 (float) or 64 (double).
void *oracle_create(const mrlbm_case_desc *d, int bits) {
    if (!d || d->nx <= 0 || d->ny <= 0 || d->nz <= 0 || d->nx % 8 || d->ny % 8 || d->nz % 4) {
        g_err = "bad descriptor (grid must be positive multiples of 8 x 8 x 4)";
        return nullptr;
    }
    const float om = reference_omega(*d);
    if (!(om > 0.f && om < 2.f)) {
        g_err = "bad descriptor: no Reynolds number and no relaxation rate in (0, 2)";
        return nullptr;
    }
    void *o = bits == 32 ? make<float>(d) : make<double>(d);
    if (!o) return nullptr;
    return new Any{bits == 32 ? 32 : 64, o};
}

void oracle_destroy(void *p) {
    if (!p) return;
    DISPATCH(p, delete o);
    delete (Any *)p;
}

void oracle_init(void *p, int kind, const double *params) { DISPATCH(p, o->init(kind, params)); }

void oracle_step(void *p, int n, int want_force) {
    DISPATCH(p, for (int s = 0; s < n; ++s) o->do_step(want_force != 0));
}

void oracle_get_moments(void *p, double *out) {
    DISPATCH(p, for (int k = 0; k < 10; ++k) for (int64_t i = 0; i < o->n; ++i) out[k * o->n + i] = (double)o->mom[k][i]);
}

void oracle_set_moments(void *p, const double *in) {
    DISPATCH(p, for (int k = 0; k < 10; ++k) for (int64_t i = 0; i < o->n; ++i) o->mom[k][i] = (decltype(o->omega))in[k * o->n + i]);
}

void oracle_get_forces(void *p, double *out) { DISPATCH(p, std::memcpy(out, o->force, sizeof(o->force))); }

void oracle_get_node_types(void *p, uint32_t *out) { DISPATCH(p, std::memcpy(out, o->type.data(), o->n * 4)); }

void oracle_get_frozen(void *p, uint8_t *out) { DISPATCH(p, std::memcpy(out, o->frozen.data(), o->n)); }

// kind: 0 wall nodes, 1 BCFLUID nodes, 2 BCSOLID nodes
int oracle_wall_size(void *p, int w, int kind) {
    int r = 0;
    DISPATCH(p, r = (int)(kind == 2 ? o->wall[w].solid.size() : kind == 1 ? o->wall[w].fluid.size() : o->wall[w].list.size()));
    return r;
}

// what: 0 list, 1 nx, 2 ny, 3 delta, 4 in, 5 out, 6 fluid list, 7 tag in, 8 tag out, 9 solid list
void oracle_get_boundary(void *p, int w, int what, void *out) {
    DISPATCH(p, {
        const WallO &W = o->wall[w];
        switch (what) {
            case 0: std::memcpy(out, W.list.data(), W.list.size() * 8); break;
            case 1: std::memcpy(out, W.nx.data(), W.nx.size() * 4); break;
            case 2: std::memcpy(out, W.ny.data(), W.ny.size() * 4); break;
            case 3: std::memcpy(out, W.delta.data(), W.delta.size() * 4); break;
            case 4: std::memcpy(out, W.in.data(), W.in.size() * 4); break;
            case 5: std::memcpy(out, W.out.data(), W.out.size() * 4); break;
            case 6: std::memcpy(out, W.fluid.data(), W.fluid.size() * 8); break;
            case 7: std::memcpy(out, o->tag_in, 1024); break;
            case 8: std::memcpy(out, o->tag_out, 1024); break;
            case 9: std::memcpy(out, W.solid.data(), W.solid.size() * 8); break;
            default: break;
        }
    });
}

}  // extern "C"
