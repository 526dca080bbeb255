// Device math of the D3Q27 moment-representation LBM: population reconstruction from
// the 10 moments, moment evaluation from 27 populations, BGK collision in moment space,
// and the boundary closures of the planar walls and of the BCFLUID nodes.
//
// Reference (paths inside sakthi-lbm/MRLBM_3D_CUDA):
//   pop_reconstruction   MRLBM_3D/src/core/D3Q27/second_order/reconstruction.cuh:5-60
//   evaluate_moments     MRLBM_3D/src/core/D3Q27/eval_moments.cuh:5-22
//   moment_collision     MRLBM_3D/src/solver/mlbm.cu:3-16
//   boundary_condition   MRLBM_3D/src/cases/cylinder/boundaries.cuh:201-843
//   update_neumaan_*     MRLBM_3D/src/cases/cylinder/boundaries.cuh:96-199
//   fluid_boundary_condition  MRLBM_3D/src/cases/cylinder/boundaries.cuh:845-1037
//   evaluate_incoming_moments_rotated  MRLBM_3D/src/boundary/curvedLBM.cu:5-59
// The arithmetic is arranged for the GB300 issue budget (shared sub-sums, pair sums);
// the closures keep the reference's formulas (they are the published solutions of the
// moment-based boundary method) written once per symmetry class with sign factors.
#pragma once

#include <cstdint>

#include "lattice_tables.h"

namespace mrlbm {

struct Mom {
    float rho;  // full density (not the stored deviation)
    float ux, uy, uz;
    float mxx, myy, mzz, mxy, mxz, myz;
};

// f_q = w_q rho [1 + 3 c.u + 4.5 (c_a c_b - delta_ab / 3) m_ab], second-order Hermite,
// as even part +- odd part: w_q rho E_q +- 3 w_q rho (c.u), with E_q built by FMAs from
// p0 = 1 - 1.5 tr(m).  Every FMA is written out (__fmaf_rn) and every product that must not
// fuse goes through __fmul_rn: the owner and the rim copies of this function keep different
// subsets of the populations, and free contraction made the two round differently.
// The Hermite factors 3 (u), 1.5, 4.5 and 9 (m) are parameters so that moments stored with a
// scale (16-bit storage) can be rebuilt without unscaling them first: pass 3 / s_u, 1.5 / s_m,
// 4.5 / s_m and 9 / s_m with the stored u and m.
__device__ __forceinline__ void reconstruct_h(const Mom &m, float h3, float h15, float h45, float h9, float f[27]) {
    const float t = __fadd_rn(__fadd_rn(m.mxx, m.myy), m.mzz);
    const float p0 = __fmaf_rn(-h15, t, 1.0f);
    const float ax = __fmaf_rn(h45, m.mxx, p0), ay = __fmaf_rn(h45, m.myy, p0), az = __fmaf_rn(h45, m.mzz, p0);
    const float r1 = __fmul_rn(m.rho, kW1), r2 = __fmul_rn(m.rho, kW2), r3 = __fmul_rn(m.rho, kW3);
    const float q1 = __fmul_rn(h3, r1), q2 = __fmul_rn(h3, r2), q3 = __fmul_rn(h3, r3);
    const float n2 = __fmul_rn(h9, r2), n3 = __fmul_rn(h9, r3);
    f[0] = __fmul_rn(__fmul_rn(m.rho, kW0), p0);
    {
        const float ex = __fmul_rn(r1, ax), ey = __fmul_rn(r1, ay), ez = __fmul_rn(r1, az);
        f[1] = __fmaf_rn(q1, m.ux, ex);
        f[2] = __fmaf_rn(-q1, m.ux, ex);
        f[3] = __fmaf_rn(q1, m.uy, ey);
        f[4] = __fmaf_rn(-q1, m.uy, ey);
        f[5] = __fmaf_rn(q1, m.uz, ez);
        f[6] = __fmaf_rn(-q1, m.uz, ez);
    }
    const float upp = __fadd_rn(m.ux, m.uy), upm = __fsub_rn(m.ux, m.uy);
    {
        const float b = __fmul_rn(r2, __fmaf_rn(h45, m.myy, ax));
        const float cp = __fmaf_rn(n2, m.mxy, b), cm = __fmaf_rn(-n2, m.mxy, b);
        f[7] = __fmaf_rn(q2, upp, cp);
        f[8] = __fmaf_rn(-q2, upp, cp);
        f[13] = __fmaf_rn(q2, upm, cm);
        f[14] = __fmaf_rn(-q2, upm, cm);
    }
    {
        const float b = __fmul_rn(r2, __fmaf_rn(h45, m.mzz, ax));
        const float cp = __fmaf_rn(n2, m.mxz, b), cm = __fmaf_rn(-n2, m.mxz, b);
        const float sp = __fadd_rn(m.ux, m.uz), sm = __fsub_rn(m.ux, m.uz);
        f[9] = __fmaf_rn(q2, sp, cp);
        f[10] = __fmaf_rn(-q2, sp, cp);
        f[15] = __fmaf_rn(q2, sm, cm);
        f[16] = __fmaf_rn(-q2, sm, cm);
    }
    {
        const float b = __fmul_rn(r2, __fmaf_rn(h45, m.mzz, ay));
        const float cp = __fmaf_rn(n2, m.myz, b), cm = __fmaf_rn(-n2, m.myz, b);
        const float sp = __fadd_rn(m.uy, m.uz), sm = __fsub_rn(m.uy, m.uz);
        f[11] = __fmaf_rn(q2, sp, cp);
        f[12] = __fmaf_rn(-q2, sp, cp);
        f[17] = __fmaf_rn(q2, sm, cm);
        f[18] = __fmaf_rn(-q2, sm, cm);
    }
    {
        const float c0 = __fmul_rn(r3, __fmaf_rn(h45, t, p0));
        const float a = __fadd_rn(m.mxy, m.mxz), b = __fsub_rn(m.mxy, m.mxz);
        const float e1 = __fmaf_rn(n3, __fadd_rn(a, m.myz), c0), e2 = __fmaf_rn(n3, __fsub_rn(b, m.myz), c0);
        const float e3 = __fmaf_rn(-n3, __fadd_rn(b, m.myz), c0), e4 = __fmaf_rn(-n3, __fsub_rn(a, m.myz), c0);
        const float s1 = __fadd_rn(upp, m.uz), s2 = __fsub_rn(upp, m.uz);
        const float s3 = __fadd_rn(upm, m.uz), s4 = __fsub_rn(upm, m.uz);
        f[19] = __fmaf_rn(q3, s1, e1);
        f[20] = __fmaf_rn(-q3, s1, e1);
        f[21] = __fmaf_rn(q3, s2, e2);
        f[22] = __fmaf_rn(-q3, s2, e2);
        f[23] = __fmaf_rn(q3, s3, e3);
        f[24] = __fmaf_rn(-q3, s3, e3);
        f[26] = __fmaf_rn(q3, s4, e4);
        f[25] = __fmaf_rn(-q3, s4, e4);
    }
}

__device__ __forceinline__ void reconstruct(const Mom &m, float f[27]) { reconstruct_h(m, 3.0f, 1.5f, 4.5f, 9.0f, f); }

// rho = sum f, u = sum c f / rho, m_ab = sum c_a c_b f / rho - cs2 delta_ab, via the 13
// opposite-pair sums e and differences d.
__device__ __forceinline__ void evaluate(const float f[27], Mom &m) {
    const float e1 = f[1] + f[2], d1 = f[1] - f[2];
    const float e3 = f[3] + f[4], d3 = f[3] - f[4];
    const float e5 = f[5] + f[6], d5 = f[5] - f[6];
    const float e7 = f[7] + f[8], d7 = f[7] - f[8];
    const float e9 = f[9] + f[10], d9 = f[9] - f[10];
    const float e11 = f[11] + f[12], d11 = f[11] - f[12];
    const float e13 = f[13] + f[14], d13 = f[13] - f[14];
    const float e15 = f[15] + f[16], d15 = f[15] - f[16];
    const float e17 = f[17] + f[18], d17 = f[17] - f[18];
    const float e19 = f[19] + f[20], d19 = f[19] - f[20];
    const float e21 = f[21] + f[22], d21 = f[21] - f[22];
    const float e23 = f[23] + f[24], d23 = f[23] - f[24];
    const float e25 = f[25] + f[26], d25 = f[25] - f[26];
    const float ec = (e19 + e21) + (e23 + e25);
    const float sxx = (e1 + e7) + (e9 + e13) + e15 + ec;
    const float syy = (e3 + e7) + (e11 + e13) + e17 + ec;
    const float szz = (e5 + e9) + (e11 + e15) + e17 + ec;
    const float rho = f[0] + ((e1 + e3) + e5) + ((e7 + e9) + (e11 + e13)) + ((e15 + e17) + ec);
    const float jx = (d1 + d7) + (d9 + d13) + (d15 + d19) + (d21 + d23) - d25;
    const float jy = (d3 + d7) + (d11 - d13) + (d17 + d19) + (d21 - d23) + d25;
    const float jz = (d5 + d9) + (d11 - d15) - (d17 - d19) + (d23 - d21) + d25;
    const float sxy = (e7 - e13) + ((e19 + e21) - (e23 + e25));
    const float sxz = (e9 - e15) + ((e19 - e21) + (e23 - e25));
    const float syz = (e11 - e17) + ((e19 - e21) - (e23 - e25));
    const float inv = __frcp_rn(rho);  // correctly rounded, as 1.0f / rho
    m.rho = rho;
    m.ux = jx * inv;
    m.uy = jy * inv;
    m.uz = jz * inv;
    m.mxx = sxx * inv - kCs2;
    m.myy = syy * inv - kCs2;
    m.mzz = szz * inv - kCs2;
    m.mxy = sxy * inv;
    m.mxz = sxz * inv;
    m.myz = syz * inv;
}

// m_ab <- (1 - omega) m_ab + omega u_a u_b; rho and u are collision invariants.  The rounding order is spelled out with
// intrinsics: `a*b + c*d` has two possible FMA contractions, and leaving the choice to the
// compiler let different kernel instantiations (tile heights) round differently.
// omega_u = omega s_m / s_u^2 collides moments held with storage scales (u s_u, m s_m);
// omega_u = omega for physical moments.
__device__ __forceinline__ void collide_h(Mom &m, float omega, float omega_u) {
    const float om1 = 1.0f - omega;
    const float wx = __fmul_rn(omega_u, m.ux), wy = __fmul_rn(omega_u, m.uy), wz = __fmul_rn(omega_u, m.uz);
    m.mxx = __fmaf_rn(wx, m.ux, __fmul_rn(om1, m.mxx));
    m.myy = __fmaf_rn(wy, m.uy, __fmul_rn(om1, m.myy));
    m.mzz = __fmaf_rn(wz, m.uz, __fmul_rn(om1, m.mzz));
    m.mxy = __fmaf_rn(wx, m.uy, __fmul_rn(om1, m.mxy));
    m.mxz = __fmaf_rn(wx, m.uz, __fmul_rn(om1, m.mxz));
    m.myz = __fmaf_rn(wy, m.uz, __fmul_rn(om1, m.myz));
}

__device__ __forceinline__ void collide(Mom &m, float omega) { collide_h(m, omega, omega); }

// ---------------------------------------------------------------------------------------
// Boundary closures (rare nodes; kept out of the bulk path with __noinline__ callers).

// Walls of a planar boundary class, as bits W=1 E=2 S=4 N=8 B=16 F=32.
__device__ __forceinline__ uint32_t class_walls(uint32_t c) {
    // classes 8..33 of the reference enum, in order
    constexpr uint8_t kWalls[34] = {0, 0, 0, 0, 0, 0, 0, 0,
                                    8, 4, 2, 1, 32, 16,            // N S E W F B
                                    10, 9, 40, 24, 6, 5, 36, 20,   // NE NW NF NB SE SW SF SB
                                    34, 18, 33, 17,                // EF EB WF WB
                                    41, 25, 37, 21, 42, 26, 38, 22};  // NWF NWB SWF SWB NEF NEB SEF SEB
    return c < 34 ? kWalls[c] : 0u;
}

// Directions whose population is known after streaming at a node on walls `w`: a wall
// removes the populations that would come from outside the grid.
__device__ __forceinline__ bool known_dir(uint32_t w, int q) {
    const int cx = cxq(q), cy = cyq(q), cz = czq(q);
    return !(((w & 1u) && cx == 1) || ((w & 2u) && cx == -1) || ((w & 4u) && cy == 1) ||
             ((w & 8u) && cy == -1) || ((w & 16u) && cz == 1) || ((w & 32u) && cz == -1));
}

struct Partial {
    float rho;                 // sum over known populations
    float sxx, syy, szz;       // sum c_a^2 f (known)
    float sxy, sxz, syz;       // sum c_a c_b f (known)
};

__device__ __forceinline__ Partial known_sums(uint32_t w, const float f[27]) {
    Partial p{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 27; ++q) {
        if (!known_dir(w, q)) continue;
        const float v = f[q];
        p.rho += v;
        if (cxq(q)) p.sxx += v;
        if (cyq(q)) p.syy += v;
        if (czq(q)) p.szz += v;
        if (cxq(q) * cyq(q) > 0) p.sxy += v;
        if (cxq(q) * cyq(q) < 0) p.sxy -= v;
        if (cxq(q) * czq(q) > 0) p.sxz += v;
        if (cxq(q) * czq(q) < 0) p.sxz -= v;
        if (cyq(q) * czq(q) > 0) p.syz += v;
        if (cyq(q) * czq(q) < 0) p.syz -= v;
    }
    return p;
}

struct PlanarCtx {
    float omega;
    float u_max;
    float rho0;
    int convective;
    // pre-stream moments of the node and of its x-1 neighbour (outlet extrapolation)
    Mom self_prev;
    Mom west_prev;
};

// Zero-gradient outlet from the x-1 neighbour, optionally blended with the node itself
// by Uc = |u_x| of the neighbour (update_neumaan_density_velocity, boundaries.cuh:163-199).
__device__ __forceinline__ void outlet_rho_u(const PlanarCtx &c, Mom &o) {
    const Mom &i = c.west_prev;
    if (c.convective) {
        const Mom &b = c.self_prev;
        const float uc = sqrtf(i.ux * i.ux);
        const double w = 1.0 - (double)uc;
        o.rho = (float)(w * (double)b.rho + (double)(uc * i.rho));
        o.ux = (float)(w * (double)b.ux + (double)(uc * i.ux));
        o.uy = (float)(w * (double)b.uy + (double)(uc * i.uy));
        o.uz = (float)(w * (double)b.uz + (double)(uc * i.uz));
    } else {
        o.rho = i.rho;
        o.ux = i.ux;
        o.uy = i.uy;
        o.uz = i.uz;
    }
}

// Planar face / edge / corner closures.  Returns false for classes without one (the node
// keeps its pre-stream moments, like the reference's switch default).
__device__ __forceinline__ bool planar_closure(uint32_t cls, const float f[27], const PlanarCtx &c, Mom &o) {
    const uint32_t w = class_walls(cls);
    if (!w) return false;
    const int nw = __popc(w);
    const bool east = (w & 2u) != 0, west = (w & 1u) != 0;
    const float om = c.omega;
    if (nw == 3) {
        // corners: west corners are no-slip with rho = 216/125 rho_I, east corners extrapolate
        if (east) {
            outlet_rho_u(c, o);
        } else {
            const Partial p = known_sums(w, f);
            o.rho = 216.0f * p.rho / 125.0f;
            o.ux = o.uy = o.uz = 0.0f;
        }
        o.mxx = o.myy = o.mzz = o.mxy = o.mxz = o.myz = 0.0f;
        return true;
    }
    const Partial p = known_sums(w, f);
    const float ri = p.rho, inv = 1.0f / ri;
    if (nw == 1) {
        if (west) {  // velocity inlet u = (U, 0, 0); rho from the known populations and the
                     // pre-stream u_x (boundaries.cuh:206-229)
            const float mxy_i = p.sxy * inv, mxz_i = p.sxz * inv;
            const float u0 = c.self_prev.ux;
            o.rho = -6.0f * ri / (-5.0f + 3.0f * u0 + 3.0f * u0 * u0);
            o.ux = c.u_max;
            o.uy = o.uz = 0.0f;
            o.mxx = o.ux * o.ux;
            o.myy = o.mzz = 0.0f;
            o.mxy = 2.0f * mxy_i * ri / o.rho;
            o.mxz = 2.0f * mxz_i * ri / o.rho;
            o.myz = 0.0f;
        } else if (east) {  // outlet (boundaries.cuh:230-271)
            const float myy_i = p.syy * inv - kCs2, mzz_i = p.szz * inv - kCs2;
            const float mxy_i = p.sxy * inv, mxz_i = p.sxz * inv, myz_i = p.syz * inv;
            outlet_rho_u(c, o);
            const float r = o.rho;
            o.mxx = o.ux * o.ux;
            o.myy = (6.0f * myy_i * ri - 6.0f * mzz_i * ri + 5.0f * o.uy * o.uy * r + 5.0f * o.uz * o.uz * r) / (10.0f * r);
            o.mzz = (-6.0f * myy_i * ri + 6.0f * mzz_i * ri + 5.0f * o.uy * o.uy * r + 5.0f * o.uz * o.uz * r) / (10.0f * r);
            o.mxy = (6.0f * mxy_i * ri - o.uy * r) / (3.0f * r);
            o.mxz = (6.0f * mxz_i * ri - o.uz * r) / (3.0f * r);
            o.myz = 6.0f * myz_i * ri / (5.0f * r);
        } else {  // no-slip face normal to y (N, S) or z (F, B)
            o.rho = 6.0f * ri / 5.0f;
            o.ux = o.uy = o.uz = 0.0f;
            o.mxx = o.myy = o.mzz = 0.0f;
            const bool ynormal = (w & 12u) != 0;
            o.mxy = ynormal ? 2.0f * (p.sxy * inv) * ri / o.rho : 0.0f;
            o.mxz = ynormal ? 0.0f : 2.0f * (p.sxz * inv) * ri / o.rho;
            o.myz = 2.0f * (p.syz * inv) * ri / o.rho;
        }
        return true;
    }
    // edges: the two normal axes a < b carry m_ab; sigma = -s_a s_b, s = +1 on the max face
    const bool xa = (w & 3u) != 0, ya = (w & 12u) != 0;
    const float sa = (w & 2u) ? 1.f : ((w & 1u) ? -1.f : ((w & 8u) ? 1.f : -1.f));
    const float sb = (w & 32u) ? 1.f : ((w & 16u) ? -1.f : ((w & 8u) ? 1.f : -1.f));
    const float sigma = -sa * sb;
    float m_i, t_i;  // normal-pair moment and, for x-edges, the other normal with the tangent
    if (xa && ya) { m_i = p.sxy * inv; t_i = p.syz * inv; }
    else if (xa) { m_i = p.sxz * inv; t_i = p.syz * inv; }
    else { m_i = p.syz * inv; t_i = 0.f; }
    if (east) {
        outlet_rho_u(c, o);
    } else {
        o.rho = sigma > 0.f ? 36.0f * ri * (1.0f + m_i - m_i * om) / (24.0f + om)
                            : 36.0f * ri * (1.0f - m_i + m_i * om) / (24.0f + om);
        o.ux = o.uy = o.uz = 0.0f;
    }
    const float r = o.rho;
    const float mab = sigma > 0.f ? (36.0f * m_i * ri + r) / (9.0f * r) : (36.0f * m_i * ri - r) / (9.0f * r);
    o.mxx = o.myy = o.mzz = 0.0f;
    if (xa && ya) { o.mxy = mab; o.mxz = 0.0f; o.myz = 12.0f * t_i * ri / (5.0f * r); }
    else if (xa) { o.mxy = 0.0f; o.mxz = mab; o.myz = 12.0f * t_i * ri / (5.0f * r); }
    else { o.mxy = 0.0f; o.mxz = 0.0f; o.myz = mab; }
    return true;
}

// Incoming partial moments over `mask`, with the lattice Hermite tensors (the reference's
// d_H** tables hold c_a c_b - cs2 delta_ab in float).
struct Incoming {
    float rho, ux, uy, uz, mxx, myy, mzz, mxy, mxz, myz;
};
__device__ __forceinline__ Incoming incoming_moments(uint32_t mask, const float f[27]) {
    Incoming s{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 27; ++q) {
        if (!(mask & (1u << q))) continue;
        const float v = f[q];
        const float cx = (float)cxq(q), cy = (float)cyq(q), cz = (float)czq(q);
        s.rho += v;
        s.ux += v * cx;
        s.uy += v * cy;
        s.uz += v * cz;
        s.mxx += v * (cx * cx - kCs2);
        s.myy += v * (cy * cy - kCs2);
        s.mzz += v * (cz * cz - kCs2);
        s.mxy += v * (cx * cy);
        s.mxz += v * (cx * cz);
        s.myz += v * (cy * cz);
    }
    const float inv = 1.0f / s.rho;
    s.ux *= inv; s.uy *= inv; s.uz *= inv;
    s.mxx *= inv; s.myy *= inv; s.mzz *= inv;
    s.mxy *= inv; s.mxz *= inv; s.myz *= inv;
    return s;
}

// BCFLUID closure for the four diagonal-quadrant tags 17, 34, 68, 136 (solid octant pair
// below/above in z at (-x,-y), (+x,-y), (-x,+y), (+x,+y)).  (sx, sy) point from the solid
// quadrant into the fluid.  Returns false for other tags (moments stay pre-stream).
__device__ __forceinline__ bool bcfluid_closure(uint32_t tag, uint32_t mask, const float f[27], int strong,
                                                float omega, Mom &o) {
    float sx, sy;
    if (tag == 17u) { sx = 1.f; sy = 1.f; }
    else if (tag == 34u) { sx = -1.f; sy = 1.f; }
    else if (tag == 68u) { sx = 1.f; sy = -1.f; }
    else if (tag == 136u) { sx = -1.f; sy = -1.f; }
    else return false;
    const Incoming I = incoming_moments(mask, f);
    const float rI = I.rho, mxx = I.mxx, myy = I.myy, mzz = I.mzz, mxy = I.mxy, mxz = I.mxz, myz = I.myz;
    const float ux = I.ux, uy = I.uy, uz = I.uz;
    const float sxy = sx * sy;
    const float us = sx * ux + sy * uy;
    const float poly = 45.0f * (mxx * mxx) + 405.0f * (mxy * mxy) + 45.0f * (myy * myy) + (345.0f * sx) * myy * ux +
                       589.0f * (ux * ux) + (345.0f * sy) * myy * uy + (1467.0f * sxy) * ux * uy + 589.0f * (uy * uy) +
                       (45.0f * sxy) * mxy * (6.0f * myy + 23.0f * us) +
                       15.0f * mxx * ((18.0f * sxy) * mxy + 6.0f * myy + 23.0f * us);
    float a, b, cc;
    if (strong) {  // MassBC::Strong quadratic (boundaries.cuh:890-897 and its mirror images)
        a = -9996.0f - 206.0f * omega;
        b = -6.0f * rI *
            (12.0f * mxx * (-17.0f + 20.0f * omega) -
             17.0f * (102.0f + (36.0f * sxy) * mxy + 12.0f * myy - (5.0f * sx) * ux - (5.0f * sy) * uy) +
             omega * ((720.0f * sxy) * mxy + 240.0f * myy + 53.0f * us));
        cc = 3.0f * omega * (rI * rI) * poly;
    } else {  // MassBC::Equilibrium quadratic
        a = -9998.0f;
        b = 6.0f * rI * (1734.0f + 66.0f * mxx + (198.0f * sxy) * mxy + 66.0f * myy + (253.0f * sx) * ux + (253.0f * sy) * uy);
        cc = 3.0f * (rI * rI) * poly;
    }
    const float disc = fmaxf(b * b - 4.0f * a * cc, 0.0f);
    const float sq = sqrtf(disc);
    const float r1 = (-b + sq) / (2.0f * a), r2 = (-b - sq) / (2.0f * a);
    const float r = (r1 > 0.0f && fabsf(r1 - rI) < fabsf(r2 - rI)) ? r1 : r2;
    o.rho = r;
    o.ux = sx * (3.0f * mxx * rI + (9.0f * sxy) * mxy * rI + 3.0f * myy * rI + (20.0f * sx) * rI * ux + (3.0f * sy) * rI * uy + r) / (17.0f * r);
    o.uy = sy * (3.0f * mxx * rI + (9.0f * sxy) * mxy * rI + 3.0f * myy * rI + (3.0f * sx) * rI * ux + (20.0f * sy) * rI * uy + r) / (17.0f * r);
    o.uz = (3.0f * rI * (sx * mxz + sy * myz + 10.0f * uz)) / (29.0f * r);
    o.mxx = (57.0f * mxx * rI + (18.0f * sxy) * mxy * rI + 6.0f * myy * rI + (6.0f * sx) * rI * ux + (6.0f * sy) * rI * uy + 2.0f * r) / (51.0f * r);
    o.myy = (6.0f * mxx * rI + (18.0f * sxy) * mxy * rI + 57.0f * myy * rI + (6.0f * sx) * rI * ux + (6.0f * sy) * rI * uy + 2.0f * r) / (51.0f * r);
    o.mzz = (36.0f * mzz * rI) / (35.0f * r);
    o.mxy = sxy * (3.0f * mxx * rI + (26.0f * sxy) * mxy * rI + 3.0f * myy * rI + (3.0f * sx) * rI * ux + (3.0f * sy) * rI * uy + r) / (17.0f * r);
    o.mxz = (rI * (32.0f * mxz + (3.0f * sxy) * myz + sx * uz)) / (29.0f * r);
    o.myz = (rI * ((3.0f * sxy) * mxz + 32.0f * myz + sy * uz)) / (29.0f * r);
    return true;
}

// BCSOLID closure (z walls only) of a z-face node beside the body, tagged by the octants of its
// neighbourhood that hold bulk fluid.  The eight tags with three of the four in-domain octants
// (0x0F or 0xF0 less one bit) have a closure; the missing octant (ox, oy, oz) points into the
// body.  The known populations are the ones pulled from inside the domain (cz != oz) less the
// two sourced from the body, x + (ox, oy, 0) and x + (ox, oy, oz).  The node is held at rest
// (u = 0, mxx = myy = mzz = mxy = 0); rho, mxz and myz follow from rhoI and the incoming mxz,
// myz.  cases/cylinder/boundaries.cuh:1039-1214 spells this out as one case per tag; here the
// eight cases are one formula in px = ox oz and py = oy oz.  Returns false for other tags
// (the moments stay pre-stream).
__device__ __forceinline__ bool bcsolid_closure(uint32_t tag, const float f[27], float omega, Mom &o) {
    int miss;
    if ((tag & 0xF0u) == 0u && __popc(tag ^ 0x0Fu) == 1) miss = __ffs(tag ^ 0x0Fu) - 1;
    else if ((tag & 0x0Fu) == 0u && __popc(tag ^ 0xF0u) == 1) miss = __ffs(tag ^ 0xF0u) - 1;
    else return false;
    const int ox = (miss & 1) ? 1 : -1, oy = (miss & 2) ? 1 : -1, oz = (miss & 4) ? 1 : -1;
    float rI = 0.f, sxz = 0.f, syz = 0.f;
#pragma unroll
    for (int q = 0; q < 27; ++q) {
        const int cx = cxq(q), cy = cyq(q), cz = czq(q);
        if (cz == oz || (cx == -ox && cy == -oy)) continue;
        const float v = f[q];
        rI += v;
        if (cx * cz > 0) sxz += v;
        else if (cx * cz < 0) sxz -= v;
        if (cy * cz > 0) syz += v;
        else if (cy * cz < 0) syz -= v;
    }
    const float inv = (float)(1.0 / (double)rI);
    const float mxzI = sxz * inv, myzI = syz * inv;
    const float px = (float)(ox * oz), py = (float)(oy * oz), pxy = px * py;
    const float w1 = omega - 1.0f;
    const float r = (108.0f * (10.0f - w1 * (px * mxzI) - w1 * (py * myzI)) * rI) / (874.0f + omega);
    o.rho = r;
    o.ux = o.uy = o.uz = 0.0f;
    o.mxx = o.myy = o.mzz = o.mxy = 0.0f;
    o.mxz = (198.0f * mxzI * rI + (18.0f * pxy) * myzI * rI + px * r) / (90.0f * r);
    o.myz = ((18.0f * pxy) * mxzI * rI + 198.0f * myzI * rI + py * r) / (90.0f * r);
    return true;
}

// Incoming rho and second moments at a curved-wall node in the frame rotated to its
// normal (cos = nx, sin = ny); u is left to the wall kernel.
__device__ __forceinline__ void incoming_rotated(float nx, float ny, uint32_t mask, const float f[27], Mom &o) {
    float r = 0.f, sxx = 0.f, syy = 0.f, szz = 0.f, sxy = 0.f, sxz = 0.f, syz = 0.f;
#pragma unroll
    for (int q = 0; q < 27; ++q) {
        if (!(mask & (1u << q))) continue;
        const float cx = (float)cxq(q), cy = (float)cyq(q), cz = (float)czq(q);
        const float cxp = cx * nx + cy * ny;
        const float cyp = -cx * ny + cy * nx;
        const float czp = cz;
        const float v = f[q];
        r += v;
        sxx += v * (cxp * cxp - kCs2);
        syy += v * (cyp * cyp - kCs2);
        szz += v * (czp * czp - kCs2);
        sxy += v * (cxp * cyp);
        sxz += v * (cxp * czp);
        syz += v * (cyp * czp);
    }
    const float inv = 1.0f / r;
    o.rho = r;
    o.mxx = sxx * inv;
    o.myy = syy * inv;
    o.mzz = szz * inv;
    o.mxy = sxy * inv;
    o.mxz = sxz * inv;
    o.myz = syz * inv;
}

// Momentum and mass carried by the populations of `mask` at one node, as
// compute_forces_mass (forces.cu:3-23) forms them: the populations rebuilt from the moments in
// FP32 and summed in FP32 in direction order.  The callers take the node's incoming minus
// outgoing sums and accumulate the nodes in FP64 (the reference accumulates FP32 atomics);
// FP64 per population would cost ~200 FP64 operations per node on a part whose FP64 rate is
// a small fraction of its FP32 rate.
static __device__ __noinline__ void masked_momentum(uint32_t mask, const Mom &m, double out[4]) {
    float f[27];
    reconstruct(m, f);
    float fx = 0.f, fy = 0.f, fz = 0.f, fm = 0.f;
#pragma unroll
    for (int q = 0; q < 27; ++q) {
        if (!(mask & (1u << q))) continue;
        fx = __fadd_rn(fx, __fmul_rn(f[q], (float)cxq(q)));
        fy = __fadd_rn(fy, __fmul_rn(f[q], (float)cyq(q)));
        fz = __fadd_rn(fz, __fmul_rn(f[q], (float)czq(q)));
        fm = __fadd_rn(fm, f[q]);
    }
    out[0] = fx;
    out[1] = fy;
    out[2] = fz;
    out[3] = fm;
}

}  // namespace mrlbm
