// Host-side node classification for the curved-wall cases.
//
// Restates the reference's host setup (paths inside sakthi-lbm/MRLBM_3D_CUDA):
//   boundary_definitions           MRLBM_3D/src/cases/cylinder/boundaries.cuh:8-94
//   load_neighbors / compute_bits  MRLBM_3D/src/cases/cylinder/nodeClass.cuh:27-108
//   mark_*_solid                   cases/cylinder/nodeClass.cuh:110-125, cases/annulus/nodeClass.cuh:109-126
//   classify_boundary_nodes_*      cases/cylinder/nodeClass.cuh:138-216, cases/annulus/nodeClass.cuh:139-257
//   classify_bcfluid_nodes_*       cases/cylinder/nodeClass.cuh:218-252, cases/annulus/nodeClass.cuh:259-307
//   classify_bcsolid_nodes_*       cases/cylinder/nodeClass.cuh:254-287, cases/annulus/nodeClass.cuh:309-357
//   buildBoundaryList / assignBoundaryIndices  cases/cylinder/cylinder_helpers.cuh:49-132
//   compute_unit_vectors_boundary_nodes        cases/cylinder/cylinder_helpers.cuh:10-47
//   find_incomings_outgoings                   cases/cylinder/cylinder_helpers.cuh:134-228
//   setup_bcfluid_masks                        cases/cylinder/cylinder_helpers.cuh:230-299
//   find_active_blocks_3d + the z-blind mask test  MRLBM_3D/src/simulation.cu:174-214, solver/mlbm.cu:87-89
// The scans run in the same z, y, x order and in place, like the reference, so lists,
// indices and per-tag masks come out identical.  This file must be compiled with
// -ffp-contract=off so that the float arithmetic rounds the same on x86-64 and aarch64.
#include <cmath>
#include <cstring>

#include "lattice_tables.h"
#include "mrlbm_internal.h"

namespace mrlbm {

namespace {

// Octant b = (cx > 0) + 2 (cy > 0) + 4 (cz > 0) holds the 7 non-rest directions whose
// nonzero components all point into that octant (the reference's bit_dirs table).
struct OctantTable {
    int dirs[8][7];
    OctantTable() {
        for (int b = 0; b < 8; ++b) {
            const int s[3] = {(b & 1) ? 1 : -1, (b & 2) ? 1 : -1, (b & 4) ? 1 : -1};
            int n = 0;
            for (int q = 1; q < 27; ++q) {
                const int c[3] = {kCx[q], kCy[q], kCz[q]};
                bool ok = true;
                for (int a = 0; a < 3; ++a) ok = ok && (c[a] == 0 || c[a] == s[a]);
                if (ok) dirs[b][n++] = q;
            }
        }
    }
};
const OctantTable &octants() {
    static OctantTable t;
    return t;
}

uint32_t face_class(bool W, bool E, bool S, bool N, bool B, bool F) {
    if (N && W && F) return C_NORTH_WEST_FRONT;
    if (N && W && B) return C_NORTH_WEST_BACK;
    if (N && E && F) return C_NORTH_EAST_FRONT;
    if (N && E && B) return C_NORTH_EAST_BACK;
    if (S && W && F) return C_SOUTH_WEST_FRONT;
    if (S && W && B) return C_SOUTH_WEST_BACK;
    if (S && E && F) return C_SOUTH_EAST_FRONT;
    if (S && E && B) return C_SOUTH_EAST_BACK;
    if (N && W) return C_NORTH_WEST;
    if (N && E) return C_NORTH_EAST;
    if (N && F) return C_NORTH_FRONT;
    if (N && B) return C_NORTH_BACK;
    if (S && W) return C_SOUTH_WEST;
    if (S && E) return C_SOUTH_EAST;
    if (S && F) return C_SOUTH_FRONT;
    if (S && B) return C_SOUTH_BACK;
    if (W && F) return C_WEST_FRONT;
    if (W && B) return C_WEST_BACK;
    if (E && F) return C_EAST_FRONT;
    if (E && B) return C_EAST_BACK;
    if (N) return C_NORTH;
    if (S) return C_SOUTH;
    if (W) return C_WEST;
    if (E) return C_EAST;
    if (F) return C_FRONT;
    if (B) return C_BACK;
    return C_BULK;
}

struct Scan {
    const mrlbm_case_desc &d;
    Geometry &g;
    int64_t idx(int x, int y, int z) const { return x + (int64_t)g.nx * (y + (int64_t)g.ny * z); }
    // Class of the 27 neighbours; outside the box counts as solid, z wraps when periodic.
    void neighbours(int x, int y, int z, uint32_t out[27]) const {
        for (int q = 0; q < 27; ++q) {
            int xn = x + kCx[q], yn = y + kCy[q], zn = z + kCz[q];
            if (d.periodic[2]) {
                if (zn < 0) zn += g.nz;
                else if (zn >= g.nz) zn -= g.nz;
                if (xn < 0 || xn >= g.nx || yn < 0 || yn >= g.ny) { out[q] = C_SOLID; continue; }
            } else if (xn < 0 || xn >= g.nx || yn < 0 || yn >= g.ny || zn < 0 || zn >= g.nz) {
                out[q] = C_SOLID;
                continue;
            }
            out[q] = g.cls[idx(xn, yn, zn)];
        }
    }
    static bool any_of(const uint32_t n[27], uint32_t c) {
        for (int q = 1; q < 27; ++q)
            if (n[q] == c) return true;
        return false;
    }
    static int octant_bits(const uint32_t n[27], uint32_t c, int bits[8]) {
        int count = 0;
        for (int b = 0; b < 8; ++b) {
            bits[b] = 0;
            for (int i = 0; i < 7; ++i)
                if (n[octants().dirs[b][i]] == c) { bits[b] = 1; break; }
            count += bits[b];
        }
        return count;
    }
    float radius(int x, int y) const {
        const float dx = (float)x - d.xc;
        const float dy = (float)y - d.yc;
        return std::sqrt(dx * dx + dy * dy);
    }
};

}  // namespace

std::string classify(const mrlbm_case_desc &d, Geometry &g) {
    g.nx = d.nx;
    g.ny = d.ny;
    g.nz = d.nz;
    const int64_t n = (int64_t)d.nx * d.ny * d.nz;
    g.cls.assign(n, C_BULK);
    g.payload.assign(n, 0);
    g.frozen.assign(n, 0);
    g.stencil.assign(n, 0);
    for (auto &w : g.wall) w = WallData();
    std::memset(g.tag_in_mask, 0, sizeof(g.tag_in_mask));
    std::memset(g.tag_out_mask, 0, sizeof(g.tag_out_mask));
    g.n_walls = d.geometry == MRLBM_GEOM_CYLINDER ? 1 : d.geometry == MRLBM_GEOM_ANNULUS ? 2 : 0;
    Scan s{d, g};

    // 1. domain faces, edges and corners (periodic axes get no tag)
    for (int z = 0; z < d.nz; ++z)
        for (int y = 0; y < d.ny; ++y)
            for (int x = 0; x < d.nx; ++x) {
                bool W = x == 0, E = x == d.nx - 1, S = y == 0, N = y == d.ny - 1, B = z == 0, F = z == d.nz - 1;
                if (d.periodic[0]) W = E = false;
                if (d.periodic[1]) S = N = false;
                if (d.periodic[2]) B = F = false;
                g.cls[s.idx(x, y, z)] = (uint8_t)face_class(W, E, S, N, B, F);
            }
    if (g.n_walls == 0) return "";

    // 2. solid region (radius in float, like the reference's host loops)
    const float r_in = 0.5f * d.d_wall[0];
    const float r_out = 0.5f * d.d_wall[1];
    const float r_mid = (float)(0.5 * (double)(float)(r_in + r_out));
    for (int z = 0; z < d.nz; ++z)
        for (int y = 0; y < d.ny; ++y)
            for (int x = 0; x < d.nx; ++x) {
                const float r = s.radius(x, y);
                const bool solid = d.geometry == MRLBM_GEOM_CYLINDER ? (r <= r_in) : (r <= r_in || r >= r_out);
                if (solid) g.cls[s.idx(x, y, z)] = C_SOLID;
            }

    const int z0 = d.periodic[2] ? 0 : 1;
    const int z1 = d.periodic[2] ? d.nz : d.nz - 1;
    const int bx0 = d.scan_box[0], bx1 = d.scan_box[1], by0 = d.scan_box[2], by1 = d.scan_box[3];
    if (bx0 < 0 || by0 < 0 || bx1 > d.nx || by1 > d.ny || bx0 >= bx1 || by0 >= by1)
        return "scan_box outside the grid";
    const bool annulus = d.geometry == MRLBM_GEOM_ANNULUS;
    uint32_t nb[27];
    int bits[8];

    // 3. wall nodes: solid nodes with fluid neighbours (and > 2 fluid octants when triangular)
    for (int z = z0; z < z1; ++z)
        for (int y = by0; y < by1; ++y)
            for (int x = bx0; x < bx1; ++x) {
                s.neighbours(x, y, z, nb);
                if (nb[0] != C_SOLID || !Scan::any_of(nb, C_BULK)) continue;
                bool take = true;
                if (d.triangular) {
                    const int cnt = Scan::octant_bits(nb, C_BULK, bits);
                    if (d.periodic[2]) take = cnt > 2;
                    else take = ((z == 0 || z == d.nz - 1) && cnt > 1) || ((z > 0 && z < d.nz - 1) && cnt > 2);
                }
                if (!take) continue;
                const bool outer = annulus && !(s.radius(x, y) < r_mid);
                g.cls[s.idx(x, y, z)] = outer ? C_OUTER : C_INNER;
            }

    // 4. BCFLUID: fluid nodes next to a deep-solid node, tagged by their solid octants
    if (d.triangular) {
        for (int z = z0; z < z1; ++z)
            for (int y = by0; y < by1; ++y)
                for (int x = bx0; x < bx1; ++x) {
                    s.neighbours(x, y, z, nb);
                    if (nb[0] != C_BULK || !Scan::any_of(nb, C_SOLID)) continue;
                    Scan::octant_bits(nb, C_SOLID, bits);
                    uint32_t tag = 0;
                    for (int b = 0; b < 8; ++b) tag |= (uint32_t)bits[b] << b;
                    const bool outer = annulus && !(s.radius(x, y) < r_mid);
                    const int64_t i = s.idx(x, y, z);
                    g.cls[i] = outer ? C_BCFLUID_OUTER : C_BCFLUID_INNER;
                    g.payload[i] = tag;
                }
    }
    // 4b. BCSOLID (z walls only): plain z-face nodes whose neighbours hold bulk fluid in fewer
    //     than four octants, tagged by those octants (nodeClass.cuh:254-287 scans the
    //     cylinder's window, annulus/nodeClass.cuh:309-357 the whole plane, like scan_box)
    if (!d.periodic[2] && d.triangular) {
        for (int z : {0, d.nz - 1})
            for (int y = by0; y < by1; ++y)
                for (int x = bx0; x < bx1; ++x) {
                    s.neighbours(x, y, z, nb);
                    if (nb[0] != C_BACK && nb[0] != C_FRONT) continue;
                    if (Scan::octant_bits(nb, C_BULK, bits) >= 4) continue;
                    uint32_t tag = 0;
                    for (int b = 0; b < 8; ++b) tag |= (uint32_t)bits[b] << b;
                    const bool outer = annulus && !(s.radius(x, y) < r_mid);
                    const int64_t i = s.idx(x, y, z);
                    g.cls[i] = outer ? C_BCSOLID_OUTER : C_BCSOLID_INNER;
                    g.payload[i] = tag;
                }
    }

    // 5. lists in lexicographic z, y, x scan order; wall index into the payload
    for (int z = 0; z < d.nz; ++z)
        for (int y = 0; y < d.ny; ++y)
            for (int x = 0; x < d.nx; ++x) {
                const int64_t i = s.idx(x, y, z);
                switch (g.cls[i]) {
                    case C_INNER: g.wall[0].list.push_back(i); break;
                    case C_OUTER: g.wall[1].list.push_back(i); break;
                    case C_BCFLUID_INNER: g.wall[0].fluid_list.push_back(i); break;
                    case C_BCFLUID_OUTER: g.wall[1].fluid_list.push_back(i); break;
                    case C_BCSOLID_INNER: g.wall[0].solid_list.push_back(i); break;
                    case C_BCSOLID_OUTER: g.wall[1].solid_list.push_back(i); break;
                    default: break;
                }
            }
    for (int w = 0; w < g.n_walls; ++w) {
        WallData &wd = g.wall[w];
        const int nbw = (int)wd.list.size();
        if (nbw <= 0) return "a curved wall has no boundary nodes";
        if (nbw >= (1 << 20)) return "too many boundary nodes for the 20-bit index";
        for (int i = 0; i < nbw; ++i) g.payload[wd.list[i]] = (uint32_t)i;
        wd.nx.resize(nbw);
        wd.ny.resize(nbw);
        wd.delta.resize(nbw);
        wd.in_mask.resize(nbw);
        wd.out_mask.resize(nbw);
        const float r_wall = 0.5f * d.d_wall[w];
        for (int i = 0; i < nbw; ++i) {
            const int64_t gi = wd.list[i];
            const int x = (int)(gi % d.nx), y = (int)((gi / d.nx) % d.ny), z = (int)(gi / ((int64_t)d.nx * d.ny));
            // unit normal and wall distance (cylinder_helpers.cuh:27-45)
            const float xb = (float)x, yb = (float)y;
            const float dx = xb - d.xc, dy = yb - d.yc;
            const float r2 = dx * dx + dy * dy;
            const float inv_r = (float)(1.0 / std::sqrt((double)r2));
            const float unx = dx * inv_r, uny = dy * inv_r;
            const float xw = d.xc + r_wall * unx, yw = d.yc + r_wall * uny;
            const float t = (xw - xb) * unx + (yw - yb) * uny;
            wd.nx[i] = unx;
            wd.ny[i] = uny;
            wd.delta[i] = t < 0.0f ? -t : t;
            // incoming / outgoing direction masks (cylinder_helpers.cuh:153-209)
            s.neighbours(x, y, z, nb);
            uint32_t in = 1u;
            for (int b = 0; b < 8; ++b) {
                bool valid = true;
                for (int k = 0; k < 7; ++k)
                    if (nb[octants().dirs[b][k]] == C_SOLID) { valid = false; break; }
                if (!valid) continue;
                for (int k = 0; k < 7; ++k) in |= 1u << kOpp[octants().dirs[b][k]];
            }
            uint32_t out = 1u;
            for (int q = 0; q < 27; ++q)
                if (in & (1u << kOpp[q])) out |= 1u << q;
            wd.in_mask[i] = in;
            wd.out_mask[i] = out;
        }
    }
    // per-tag BCFLUID masks from the first node of each tag in a wall's list; the walls run
    // inner then outer, each with a fresh "seen" table, so the outer wall's node wins for a
    // tag present on both (cylinder_helpers.cuh:230-299, annulus_kernels.cu:37-38)
    if (d.triangular) {
        for (int w = 0; w < g.n_walls; ++w) {
            bool done[256] = {false};
            for (int64_t gi : g.wall[w].fluid_list) {
                const uint32_t tag = g.payload[gi];
                if (done[tag]) continue;
                const int x = (int)(gi % d.nx), y = (int)((gi / d.nx) % d.ny), z = (int)(gi / ((int64_t)d.nx * d.ny));
                s.neighbours(x, y, z, nb);
                uint32_t in = (1u << 27) - 1;
                for (int q = 0; q < 27; ++q)
                    if (nb[q] == C_SOLID) in &= ~(1u << kOpp[q]);
                uint32_t out = 0;
                for (int q = 0; q < 27; ++q)
                    if (in & (1u << kOpp[q])) out |= 1u << q;
                g.tag_in_mask[tag] = in;
                g.tag_out_mask[tag] = out;
                done[tag] = true;
            }
        }
    }

    // 6. frozen nodes: the reference skips 8x8x4 blocks whose mask entry
    //    active[by * GX + bx] (z-blind, i.e. the bz = 0 block) marks an all-solid block.
    {
        const int gx = (d.nx + 7) / 8, gy = (d.ny + 7) / 8;
        std::vector<uint8_t> active((size_t)gx * gy, 0);
        for (int by = 0; by < gy; ++by)
            for (int bx = 0; bx < gx; ++bx) {
                bool any = false;
                for (int z = 0; z < 4 && z < d.nz && !any; ++z)
                    for (int y = by * 8; y < by * 8 + 8 && y < d.ny && !any; ++y)
                        for (int x = bx * 8; x < bx * 8 + 8 && x < d.nx; ++x)
                            if (g.cls[s.idx(x, y, z)] != C_SOLID) { any = true; break; }
                active[(size_t)by * gx + bx] = any;
            }
        for (int z = 0; z < d.nz; ++z)
            for (int y = 0; y < d.ny; ++y)
                for (int x = 0; x < d.nx; ++x)
                    g.frozen[s.idx(x, y, z)] = !active[(size_t)(y / 8) * gx + (x / 8)];
    }

    // 7. stencil nodes: every node whose post-stream moments the wall kernel reads (own
    //    node and the bilinear cells at 1, 2 and 3 lattice units along the normal), with a
    //    one-cell margin so a last-bit difference in floor() can never leave the set.
    for (int w = 0; w < g.n_walls; ++w) {
        const WallData &wd = g.wall[w];
        const float r_wall = 0.5f * d.d_wall[w];
        const float dir = (w == 1) ? -1.0f : 1.0f;
        for (size_t i = 0; i < wd.list.size(); ++i) {
            const int64_t gi = wd.list[i];
            g.stencil[gi] = 1;
            const int z = (int)(gi / ((int64_t)d.nx * d.ny));
            const double xw = d.xc + (double)r_wall * wd.nx[i], yw = d.yc + (double)r_wall * wd.ny[i];
            for (int k = 1; k <= 3; ++k) {
                const double px = xw + dir * k * wd.nx[i], py = yw + dir * k * wd.ny[i];
                const int fx = (int)std::floor(px), fy = (int)std::floor(py);
                if (fx - 1 < 0 || fy - 1 < 0 || fx + 2 >= d.nx || fy + 2 >= d.ny)
                    return "a curved-wall interpolation point falls outside the grid";
                for (int yy = fy - 1; yy <= fy + 2; ++yy)
                    for (int xx = fx - 1; xx <= fx + 2; ++xx) g.stencil[s.idx(xx, yy, z)] = 1;
            }
        }
    }
    return "";
}

std::string derive(mrlbm_case_desc &d, Derived &out) {
    if (d.omega <= 0.0f) {
        // Float / double mix of the reference's constexpr chains:
        //   cylinder  VISC = U_MAX * D_WALL / RE; TAU = 0.5 + 3.0 * VISC   (cylinder/constants.cuh:52-54)
        //   annulus   VISC = U_REL * GAP / RE;    TAU = 0.5 + as2 * VISC   (annulus/constants.cuh:73-81)
        float visc;
        double tau;
        if (d.geometry == MRLBM_GEOM_ANNULUS) {
            const float r_in = 0.5f * d.d_wall[0], r_out = 0.5f * d.d_wall[1];
            const float du = d.wall_u[0][1] - d.wall_u[1][1];
            const float u_rel = du < 0.0f ? -du : du;
            const float gap = r_out - r_in;
            visc = u_rel * gap / d.re;
            tau = 0.5 + (double)(3.0f * visc);
        } else {
            const float l = d.geometry == MRLBM_GEOM_CYLINDER ? d.d_wall[0] : d.length;
            visc = d.u_max * l / d.re;
            tau = 0.5 + 3.0 * (double)visc;
        }
        const float tau_f = (float)tau;
        d.omega = (float)(1.0 / (double)tau_f);
    }
    out.omega = d.omega;
    out.tau = (float)(1.0 / (double)d.omega);
    // stability guards of initializeLBM.cuh:8-26, as errors
    if (!(out.tau > 0.5f && out.tau < 2.5f)) return "tau out of the stable LBM range (0.5, 2.5)";
    const double ma = (double)d.u_max / std::sqrt(1.0 / 3.0);
    if (ma > 0.33) return "Mach number too high (U / cs > 0.33)";
    return "";
}

}  // namespace mrlbm
