// Fused MR-LBM time step: stream + moment evaluation / boundary closure + collision in one
// pass over HBM (one moment read, one moment write per node).
//
// Replaces the reference's two full-grid kernels and their population halo
// (paths inside sakthi-lbm/MRLBM_3D_CUDA):
//   streaming_and_evaluate_Mom  MRLBM_3D/src/solver/mlbm.cu:83-164
//   collision_halo_update       MRLBM_3D/src/solver/mlbm.cu:186-242
//   pop_load_from_halo / pop_save_to_halo / save_pop / streaming
//                               MRLBM_3D/src/core/D3Q27/halo_interface.cuh:5-201, core/streaming.cuh:6-35
// The reference streams populations rebuilt from the stored (post-collision) moments:
// f_q(x) = R(M(x - c_q))_q on a grid that wraps in every axis, then evaluates moments or a
// boundary closure, then collides.  Here each CTA owns a 32 x TY column of nodes and marches
// along z.  For every plane it rebuilds the populations of the column plus a one-node rim
// (neighbour moments read through L2) into shared-memory ring buffers split by c_z, so a
// node's 27 pulled populations come from planes z-1, z, z+1 without any population array in
// HBM.  Post-collision moments go to the second ping-pong buffer.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

#include "mrlbm_internal.h"
#include "storage.cuh"

namespace mrlbm {
namespace {

// Populations exchanged through shared memory, split by c_z (the three c = (0,0,c_z)
// populations stay in registers of the column's owner thread).
// Eight 5-bit direction indices per class packed in one constant:
//   up   (c_z = +1, pulled from plane z-1): 9, 11, 16, 18, 19, 22, 23, 25
//   flat (c_z =  0, pulled from plane z):   1, 2, 3, 4, 7, 8, 13, 14
//   down (c_z = -1, pulled from plane z+1): 10, 12, 15, 17, 20, 21, 24, 26
constexpr unsigned long long pack5(int a, int b, int c, int d, int e, int f, int g, int h) {
    return (unsigned long long)a | (unsigned long long)b << 5 | (unsigned long long)c << 10 |
           (unsigned long long)d << 15 | (unsigned long long)e << 20 | (unsigned long long)f << 25 |
           (unsigned long long)g << 30 | (unsigned long long)h << 35;
}
constexpr unsigned long long kUpBits = pack5(9, 11, 16, 18, 19, 22, 23, 25);
constexpr unsigned long long kFlBits = pack5(1, 2, 3, 4, 7, 8, 13, 14);
constexpr unsigned long long kDnBits = pack5(10, 12, 15, 17, 20, 21, 24, 26);
__host__ __device__ constexpr int hUp(int j) { return (int)((kUpBits >> (5 * j)) & 31ull); }
__host__ __device__ constexpr int hFl(int j) { return (int)((kFlBits >> (5 * j)) & 31ull); }
__host__ __device__ constexpr int hDn(int j) { return (int)((kDnBits >> (5 * j)) & 31ull); }

template <int TY>
struct Geo {
    static constexpr int NOWN = TILE_X * TY;    // owner threads: one per column, one warp per row
    static constexpr int NR = 2 * TILE_X + 2 * TY + 4;  // rim columns
    static constexpr int NRW = (NR + 31) / 32;  // dedicated rim warps
    static constexpr int NTH = NOWN + 32 * NRW;
    static constexpr int W = TILE_X + 2;        // shared-memory row pitch (column + rim)
    static constexpr int NCOL = W * (TY + 2);   // columns incl. rim
    static constexpr int PLANE = 8 * NCOL;      // floats of one 8-population plane buffer
    static constexpr int NUP = 4, NFL = 3, NDN = 2;  // ring depths (rim warps run one plane ahead)
    static constexpr int SMEM = (NUP + NFL + NDN) * PLANE * 4;
    static constexpr int MINB = TY == 4 ? 3 : (TY == 8 ? 2 : 1);  // resident CTAs per SM targeted
};

constexpr bool need_dir(int q, int rcx, int rcy) {
    return (rcx == 0 || cxq(q) == rcx) && (rcy == 0 || cyq(q) == rcy);
}

// Rebuild the populations of one rim column and store the ones the tile pulls from it
// (rcx, rcy: the c_x / c_y a population must have to enter the tile from this rim side).
template <typename S, int RCX, int RCY, int TY>
__device__ __forceinline__ void rim_store(const Raw<S> &raw, float rho0, const StorageScale &sc, float *up,
                                          float *fl, float *dn, int col) {
    constexpr int NC = Geo<TY>::NCOL;
    float f[27];
    rebuild<S>(raw, rho0, sc, f);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (need_dir(hUp(j), RCX, RCY)) up[j * NC + col] = f[hUp(j)];
        if (need_dir(hFl(j), RCX, RCY)) fl[j * NC + col] = f[hFl(j)];
        if (need_dir(hDn(j), RCX, RCY)) dn[j * NC + col] = f[hDn(j)];
    }
}

// Pulled population q of the owner node, read from the ring buffer of its c_z class.
template <int Q, int TY>
__device__ __forceinline__ float pull(const float *up, const float *fl, const float *dn, int col) {
    constexpr int NC = Geo<TY>::NCOL, W = Geo<TY>::W;
    constexpr int off = -cyq(Q) * W - cxq(Q);
    if constexpr (czq(Q) == 1) {
        constexpr int j = Q == 9 ? 0 : Q == 11 ? 1 : Q == 16 ? 2 : Q == 18 ? 3 : Q == 19 ? 4 : Q == 22 ? 5 : Q == 23 ? 6 : 7;
        return up[j * NC + col + off];
    } else if constexpr (czq(Q) == 0) {
        constexpr int j = Q == 1 ? 0 : Q == 2 ? 1 : Q == 3 ? 2 : Q == 4 ? 3 : Q == 7 ? 4 : Q == 8 ? 5 : Q == 13 ? 6 : 7;
        return fl[j * NC + col + off];
    } else {
        constexpr int j = Q == 10 ? 0 : Q == 12 ? 1 : Q == 15 ? 2 : Q == 17 ? 3 : Q == 20 ? 4 : Q == 21 ? 5 : Q == 24 ? 6 : 7;
        return dn[j * NC + col + off];
    }
}

// Zeroth, first and second (c_x, c_y) sums of the 3 x 3 populations of one c_z class, from
// row sums (by c_y) and column sums (by c_x): 19 additions instead of one per term.
struct ClassSums {
    float s0, sx, sy, sxx, syy, sxy;
};
__device__ __forceinline__ ClassSums class_sums(float mm, float m0, float mp, float zm, float zz, float zp, float pm,
                                                float p0, float pp) {
    // arguments: f(c_x, c_y) with m = -1, z = 0, p = +1, named <c_x><c_y>
    const float rp = (mp + zp) + pp, r0 = (m0 + zz) + p0, rm = (mm + zm) + pm;  // by c_y = +1, 0, -1
    const float cp = (pm + p0) + pp, cm = (mm + m0) + mp;                       // by c_x = +1, -1
    ClassSums s;
    s.s0 = (rp + r0) + rm;
    s.sx = cp - cm;
    s.sxx = cp + cm;
    s.sy = rp - rm;
    s.syy = rp + rm;
    s.sxy = (pp + mm) - (pm + mp);
    return s;
}

// Packed FP32 (sm_100+ add / sub .rn.f32x2): one instruction, two independently IEEE-rounded
// lanes, so a packed sum gives bit for bit the two scalar sums.
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    unsigned long long ra, rb, rd;
    memcpy(&ra, &a, 8);
    memcpy(&rb, &b, 8);
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(rd) : "l"(ra), "l"(rb));
    float2 d;
    memcpy(&d, &rd, 8);
    return d;
}

// class_sums of two classes at once (lane x, lane y), the same operations in the same order
struct ClassSums2 {
    float2 s0, sx, sy, sxx, syy, sxy;
};
__device__ __forceinline__ ClassSums2 class_sums2(float2 mm, float2 m0, float2 mp, float2 zm, float2 zz, float2 zp,
                                                  float2 pm, float2 p0, float2 pp) {
    const float2 rp = add2(add2(mp, zp), pp), r0 = add2(add2(m0, zz), p0), rm = add2(add2(mm, zm), pm);
    const float2 cp = add2(add2(pm, p0), pp), cm = add2(add2(mm, m0), mp);
    ClassSums2 s;
    s.s0 = add2(add2(rp, r0), rm);
    s.sx = sub2(cp, cm);
    s.sxx = add2(cp, cm);
    s.sy = sub2(rp, rm);
    s.syy = add2(rp, rm);
    s.sxy = sub2(add2(pp, mm), add2(pm, mp));
    return s;
}

// Gather the pulled populations of the owner node and evaluate its moments on the fly,
// class by class (c_z = +1 from plane z-1, 0 from z, -1 from z+1); the c_z = +1 and c_z = 0
// classes share packed sums (lane x: +1, lane y: 0).
// SCALED: u and the second moments come out multiplied by the storage scales su and sm.
template <int TY, bool SCALED = false>
__device__ __forceinline__ void gather_evaluate(const float *up, const float *fl, const float *dn, int col, float f0,
                                                float f5, float f6, Mom &m, float su = 1.0f, float sm = 1.0f) {
#define MRLBM_P(q) pull<q, TY>(up, fl, dn, col)
#define MRLBM_P2(a, b) make_float2(MRLBM_P(a), MRLBM_P(b))
    // (c_x, c_y) = (-1,-1), (-1,0), (-1,1), (0,-1), (0,0), (0,1), (1,-1), (1,0), (1,1):
    // c_z = +1: 22, 16, 25, 18, 5, 11, 23, 9, 19;  c_z = 0: 8, 2, 14, 4, 0, 3, 13, 1, 7
    const ClassSums2 uc = class_sums2(MRLBM_P2(22, 8), MRLBM_P2(16, 2), MRLBM_P2(25, 14), MRLBM_P2(18, 4),
                                      make_float2(f5, f0), MRLBM_P2(11, 3), MRLBM_P2(23, 13), MRLBM_P2(9, 1),
                                      MRLBM_P2(19, 7));
    // c_z = -1: 20, 10, 24, 12, 6, 17, 26, 15, 21
    const ClassSums d = class_sums(MRLBM_P(20), MRLBM_P(10), MRLBM_P(24), MRLBM_P(12), f6, MRLBM_P(17), MRLBM_P(26),
                                   MRLBM_P(15), MRLBM_P(21));
#undef MRLBM_P2
#undef MRLBM_P
    const float rho = (uc.s0.x + uc.s0.y) + d.s0;
    const float inv = __frcp_rn(rho);  // correctly rounded, as 1.0f / rho
    const float iu = SCALED ? __fmul_rn(inv, su) : inv, im = SCALED ? __fmul_rn(inv, sm) : inv;
    const float cs = SCALED ? __fmul_rn(-kCs2, sm) : -kCs2;
    m.rho = rho;
    m.ux = ((uc.sx.x + uc.sx.y) + d.sx) * iu;
    m.uy = ((uc.sy.x + uc.sy.y) + d.sy) * iu;
    m.uz = (uc.s0.x - d.s0) * iu;
    m.mxx = __fmaf_rn((uc.sxx.x + uc.sxx.y) + d.sxx, im, cs);
    m.myy = __fmaf_rn((uc.syy.x + uc.syy.y) + d.syy, im, cs);
    m.mzz = __fmaf_rn(uc.s0.x + d.s0, im, cs);
    m.mxy = ((uc.sxy.x + uc.sxy.y) + d.sxy) * im;
    m.mxz = (uc.sx.x - d.sx) * im;
    m.myz = (uc.sy.x - d.sy) * im;
}

template <int TY>
__device__ __forceinline__ void gather_all(const float *up, const float *fl, const float *dn, int col, float f0,
                                           float f5, float f6, float *f) {
    f[0] = f0;
    f[5] = f5;
    f[6] = f6;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        f[hUp(j)] = up[j * Geo<TY>::NCOL + col - cyq(hUp(j)) * Geo<TY>::W - cxq(hUp(j))];
        f[hFl(j)] = fl[j * Geo<TY>::NCOL + col - cyq(hFl(j)) * Geo<TY>::W - cxq(hFl(j))];
        f[hDn(j)] = dn[j * Geo<TY>::NCOL + col - cyq(hDn(j)) * Geo<TY>::W - cxq(hDn(j))];
    }
}

// Rebuild the own-column populations of plane p from raw stored moments into the rings.
template <typename S, int TY>
__device__ __forceinline__ void arrive_own(const Raw<S> &raw, float rho0, const StorageScale &sc, float *up,
                                           float *fl, float *dn, int col, float &c0, float &c5, float &c6) {
    float f[27];
    rebuild<S>(raw, rho0, sc, f);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        up[j * Geo<TY>::NCOL + col] = f[hUp(j)];
        fl[j * Geo<TY>::NCOL + col] = f[hFl(j)];
        dn[j * Geo<TY>::NCOL + col] = f[hDn(j)];
    }
    c0 = f[0];
    c5 = f[5];
    c6 = f[6];
}

template <typename S, int TY>
__device__ __forceinline__ void arrive_rim(const Raw<S> &raw, float rho0, const StorageScale &sc, int side, float *up,
                                           float *fl, float *dn, int rcol) {
    switch (side) {
        case 0: rim_store<S, 0, 1, TY>(raw, rho0, sc, up, fl, dn, rcol); break;
        case 1: rim_store<S, 0, -1, TY>(raw, rho0, sc, up, fl, dn, rcol); break;
        case 2: rim_store<S, 1, 0, TY>(raw, rho0, sc, up, fl, dn, rcol); break;
        case 3: rim_store<S, -1, 0, TY>(raw, rho0, sc, up, fl, dn, rcol); break;
        case 4: rim_store<S, 1, 1, TY>(raw, rho0, sc, up, fl, dn, rcol); break;
        case 5: rim_store<S, -1, 1, TY>(raw, rho0, sc, up, fl, dn, rcol); break;
        case 6: rim_store<S, 1, -1, TY>(raw, rho0, sc, up, fl, dn, rcol); break;
        default: rim_store<S, -1, -1, TY>(raw, rho0, sc, up, fl, dn, rcol); break;
    }
}

// Post-stream (pre-collision) moments of a wall-stencil node into its side-buffer entry, the
// snapshot the wall kernel interpolates from (the node-list kernel writes the same for the
// marked nodes it handles); iu / im undo the storage scales of the 16-bit emit.
template <int TY>
__device__ __forceinline__ void snapshot_t(float *side, int slot, int x, int y, int z, int x0, int y0, int nz,
                                           const Mom &m, float rho0, float iu, float im) {
    float *e = side + side_index(slot, x, y, z, x0, y0, nz, TILE_X, TY) * 16;
    e[0] = m.rho - rho0;
    e[1] = m.ux * iu; e[2] = m.uy * iu; e[3] = m.uz * iu;
    e[4] = m.mxx * im; e[5] = m.myy * im; e[6] = m.mzz * im;
    e[7] = m.mxy * im; e[8] = m.mxz * im; e[9] = m.myz * im;
}

// Named CTA barriers (PTX bar.sync / bar.arrive; id 0 is __syncthreads).  A generation
// completes when `n` threads (whole warps) have arrived; bar.arrive does not wait.
__device__ __forceinline__ void nb_sync(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }
__device__ __forceinline__ void nb_arrive(int id, int n) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// SPECIAL = false: every node of every item is a plain bulk node (no node words are read).
// FULL = true: every tile is a whole 32 x TY tile (nx % 32 == 0, ny % TY == 0), so the
// ragged-edge predicates fold away and the owner branches are warp-uniform.
//
// Warp roles and schedule per work item (planes indexed k = 0 .. L+1 from zs-1, L = ze-zs):
//   owner warps (one per tile row):  rebuild own columns of plane k; for k >= 2 wait FULL(k),
//       emit plane k-1 (reads up(k-2), flat(k-1), down(k)), then signal DONE(k) if a rim
//       iteration k+2 will wait for it;
//   rim warps:  for k >= 4 wait DONE(k-2); rebuild the rim columns of plane k; for k >= 2
//       signal FULL(k).
// Plane k's buffers live in ring slots up[k%4], flat[k%3], down[k%2]; their previous
// occupants (plane k-4 / k-3 / k-2) are last read by the emit of iteration k-2, which both
// roles wait for before writing (owners through FULL(k-1)).  FULL(k) / DONE(k) use barrier ids
// 1 + (k&1) / 3 + (k&1); a role can run at most one generation ahead on an id, so
// consecutive generations never mix.  Counts are always the whole CTA (owner arrivals +
// rim arrivals), so the rim work of the next plane overlaps the owners' emit.
template <typename S, int TY, bool SPECIAL, bool BATCH, bool FULL>
__global__ void __launch_bounds__(Geo<TY>::NTH, Geo<TY>::MINB)
    step_kernel(const StepArgs *__restrict__ ga, const BatchArgs *__restrict__ ba, const int parity,
                double *__restrict__ diag_part) {
    using G = Geo<TY>;
    extern __shared__ float smem[];
    __shared__ double red[2][TY];
    // per-case values: fixed for a single case, reloaded per work item in a batch
    const S *__restrict__ src = nullptr;
    S *__restrict__ dst = nullptr;
    int nxb = 0, nx = 0, ny = 0, nz = 0, lz = 0, tiles_x = 0;
    const int32_t *__restrict__ tile_slot = nullptr;
    const uint32_t *__restrict__ word = nullptr;
    float *__restrict__ popbuf = nullptr;
    float *__restrict__ side = nullptr;  // wall-stencil snapshots of special tiles
    int n_pop = 0;
    const int32_t *__restrict__ row_base = nullptr;
    float omega = 1.f, rho0 = 1.f;
    StorageScale sc;
    int64_t plane = 0, zst = 0;  // lexicographic plane (node words), storage elements per z plane
    bool sr_on = false;          // stochastic rounding of 16-bit stores
    uint32_t sr_seed = 0u;
    float omega_u = 1.f;         // omega s_m / s_u^2: collision of scaled 16-bit moments
    auto load_case = [&](const StepArgs *__restrict__ c) {
        src = (const S *)c->m[parity];
        dst = (S *)c->m[parity ^ 1];
        nxb = c->nxb;
        nx = c->nx;
        ny = c->ny;
        nz = c->nz;
        lz = c->lz;
        tiles_x = c->tiles_x;
        tile_slot = c->tile_slot;
        word = c->word;
        popbuf = c->popbuf;
        side = c->side;
        n_pop = c->n_list_pop;
        row_base = c->row_base;
        omega = c->omega;
        rho0 = c->rho0;
        sc = c->sc;
        plane = (int64_t)nx * ny;
        zst = (int64_t)ny * nxb * StorageLayout<S>::per_node * kXBlock;
        if constexpr (kScaled<S>) {
            sr_on = c->sr_step != nullptr;
            sr_seed = sr_on ? sr_step_seed(*c->sr_step) : 0u;
            omega_u = c->omega * (c->sc.s[2] * (c->sc.is[1] * c->sc.is[1]));
        }
    };
    if constexpr (!BATCH) load_case(ga);
    const int n_items = BATCH ? ba->n_items : ga->n_items;
    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    const bool owner = tid < G::NOWN;
    const bool diag = diag_part != nullptr;
    float *const up_base = smem;
    float *const fl_base = smem + G::NUP * G::PLANE;
    float *const dn_base = smem + (G::NUP + G::NFL) * G::PLANE;
    double dmD = 0.0, deD = 0.0;

    // Work items: the first gridDim.x go by block index, the rest are claimed on demand from
    // a counter zeroed before every launch, so CTAs that finish early take more (no static
    // last-wave imbalance).  Without a counter the CTAs stride through the list.
    int *const work = BATCH ? ba->work_counter : ga->work_counter;
    __shared__ int s_next;
    for (int it = blockIdx.x; it < n_items;) {
        int item;
        if constexpr (BATCH) {
            const int2 e = ba->items[it];
            load_case(ba->cases[e.x]);
            item = e.y;
        } else {
            item = ga->items[it];
        }
        const int tile = item & 0xFFFFF, seg = item >> 20;
        const int tix = tile % tiles_x, tiy = tile / tiles_x;
        const int x0 = tix * TILE_X, y0 = tiy * TY;
        const int w = FULL ? TILE_X : min(TILE_X, nx - x0), h = FULL ? TY : min(TY, ny - y0);
        const int zs = seg * lz, ze = min(zs + lz, nz);
        const int last = ze - zs + 1;  // last plane index k
        const int slot = (SPECIAL && tile_slot) ? tile_slot[tile] : -1;
        const bool own = owner && (FULL || (tx < w && ty < h));
        const int x = x0 + tx, y = y0 + ty;
        const int col = (ty + 1) * G::W + (tx + 1);
        // the column this thread loads and rebuilds: its own, or a rim column for rim warps
        int rside = -1, ccol = col;
        int64_t cxy = 0;
        bool active = own;
        if (own) {
            cxy = aos_at<S>(x, y, 0, nxb, ny);
        } else if (!owner) {
            int rx, ry, sd;
            const int r = tid - G::NOWN;
            if (r < TILE_X) { rx = r; ry = -1; sd = 0; }
            else if (r < 2 * TILE_X) { rx = r - TILE_X; ry = h; sd = 1; }
            else if (r < 2 * TILE_X + TY) { rx = -1; ry = r - 2 * TILE_X; sd = 2; }
            else if (r < 2 * TILE_X + 2 * TY) { rx = w; ry = r - 2 * TILE_X - TY; sd = 3; }
            else if (r < G::NR) {
                const int k = r - 2 * TILE_X - 2 * TY;
                rx = (k & 1) ? w : -1;
                ry = (k & 2) ? h : -1;
                sd = 4 + k;
            } else { rx = 0; ry = 0; sd = -1; }
            const bool valid = sd >= 0 && ((sd == 0 || sd == 1) ? rx < w : ((sd == 2 || sd == 3) ? ry < h : true));
            if (valid) {
                rside = sd;
                ccol = (ry + 1) * G::W + (rx + 1);
                int gx = x0 + rx, gy = y0 + ry;
                gx = gx < 0 ? gx + nx : (gx >= nx ? gx - nx : gx);
                gy = gy < 0 ? gy + ny : (gy >= ny ? gy - ny : gy);
                cxy = aos_at<S>(gx, gy, 0, nxb, ny);
                active = true;
            }
        }

        // raw moments of planes k (being rebuilt) and k+1 (in flight); the two buffers swap
        // roles every plane, so the plane loops are unrolled by two
        Raw<S> pa, pb;
        const int zm = zs == 0 ? nz - 1 : zs - 1;
        if (active) load_words<S>(src, cxy + (int64_t)zm * zst, pa);
        int zn = zs;  // plane of the next prefetch (wrapped)
        int64_t loff = cxy + (int64_t)zs * zst;  // its storage offset, advanced per plane
        int64_t soff = loff;                      // storage offset of the next emitted plane
        const int64_t wrap = (int64_t)nz * zst;
        int k3 = 0, k4 = 0;  // k % 3, k % 4

        if (owner) {
            float c0 = 0.f, c5 = 0.f, c6 = 0.f;   // own-column rest / up / down populations of plane k
            float p0 = 0.f, p5 = 0.f, pp5 = 0.f;  // f0(k-1), f5(k-1), f5(k-2)
            float dm = 0.f, de = 0.f;
            // special tiles: node word and list row base of the plane emitted two planes later,
            // one queue slot per plane parity
            uint32_t wqa = 0u, wqb = 0u;
            int rqa = 0, rqb = 0;
            const unsigned row_mask = w >= 32 ? 0xffffffffu : ((1u << w) - 1u);
            // wq / rq: this parity's queue slot (the plane emitted now, refilled for k + 2); wo: the
            // other slot, which holds the word of the plane rebuilt now
            auto owner_plane = [&](const int k, const Raw<S> &cur, Raw<S> &nxt, uint32_t &wq, int &rq,
                                   const uint32_t wo) {
                float *up = up_base + k4 * G::PLANE;
                float *flt = fl_base + k3 * G::PLANE;
                float *dn = dn_base + (k & 1) * G::PLANE;
                uint32_t wnew = 0u;
                int rnew = 0;
                if constexpr (SPECIAL) {
                    if (slot >= 0 && own && k + 2 <= last) {
                        const int zq = zs + k;
                        wnew = word[(int64_t)x + (int64_t)nx * y + (int64_t)zq * plane];
                        rnew = row_base[((int64_t)slot * nz + zq) * TY + ty];
                    }
                }
                if (own) {
                    if (k < last) {
                        load_words<S>(src, loff, nxt);
                        loff += zst;
                        if (++zn == nz) {
                            zn = 0;
                            loff -= wrap;
                        }
                    }
                    arrive_own<S, TY>(cur, rho0, sc, up, flt, dn, col, c0, c5, c6);
                    if constexpr (SPECIAL) {
                        // a solid node of an updated block in the plane rebuilt now (z = zs + k - 1,
                        // one this segment emits) keeps its stored moments, collided (the reference
                        // collides every node of an active block): finished here from the words
                        // in registers, before the emit would need them reloaded
                        if (k >= 1 && k < last && (wo & NW_CLASS_MASK) == C_SOLID && !(wo & NW_FROZEN)) {
                            Mom m = decode_words<S>(cur, rho0, sc);
                            const int zr = zs + k - 1;
                            const int64_t ar = k >= 2 ? soff + zst : soff;  // soff: plane zs + k - 2
                            if (wo & NW_STENCIL)
                                snapshot_t<TY>(side, slot, x, y, zr, x0, y0, nz, m, rho0, 1.0f, 1.0f);
                            collide(m, omega);
                            if (kScaled<S> && sr_on)
                                store_mom_sr<S>(dst, ar, m, rho0, sc, sr_key(sr_seed, x, y, zr, nx, ny));
                            else
                                store_mom<S>(dst, ar, m, rho0, sc);
                        }
                    }
                }
                if (k >= 2) {
                    nb_sync(1 + (k & 1), G::NTH);  // FULL(k): plane k complete, emits of k-1 done
                    const int z = zs + k - 2;      // emitted plane
                    if (own) {
                        const float *eup = up_base + (k4 >= 2 ? k4 - 2 : k4 + 2) * G::PLANE;  // plane k-2
                        const float *efl = fl_base + (k3 >= 1 ? k3 - 1 : 2) * G::PLANE;       // plane k-1
                        const int64_t ai = soff;
                        uint32_t wd = 0u;
                        bool exp = false;
                        unsigned bal = 0u;
                        if constexpr (SPECIAL) {
                            if (slot >= 0) {
                                wd = wq;
                                // a plain fluid node whose only mark is the wall-stencil bit is
                                // updated here, like any bulk node, plus its snapshot; every other
                                // marked node goes to the node-list kernel
                                exp = wd != 0u && wd != NW_STENCIL && !(wd & NW_FROZEN) &&
                                      (wd & NW_CLASS_MASK) != C_SOLID;
                                bal = __ballot_sync(row_mask, exp);
                            }
                        }
                        const bool snap = SPECIAL && wd == NW_STENCIL;
                        if (wd == 0u || snap) {
                            Mom m;
                            if constexpr (std::is_same<S, float>::value) {
                                gather_evaluate<TY>(eup, efl, dn, col, p0, pp5, c6, m);
                                if (snap) snapshot_t<TY>(side, slot, x, y, z, x0, y0, nz, m, rho0, 1.0f, 1.0f);
                                if (diag) {
                                    dm += m.rho - rho0;
                                    de += 0.5f * (m.ux * m.ux + m.uy * m.uy + m.uz * m.uz);
                                }
                                collide(m, omega);
                                store_mom<S>(dst, ai, m, rho0, sc);
                            } else {
                                // u and m come out with their storage scales: no unscaling on
                                // the way in (rebuild) and no scaling on the way out
                                gather_evaluate<TY, true>(eup, efl, dn, col, p0, pp5, c6, m, sc.s[1], sc.s[2]);
                                if (snap) snapshot_t<TY>(side, slot, x, y, z, x0, y0, nz, m, rho0, sc.is[1], sc.is[2]);
                                if (diag) {
                                    dm += m.rho - rho0;
                                    de += 0.5f * (m.ux * m.ux + m.uy * m.uy + m.uz * m.uz) * (sc.is[1] * sc.is[1]);
                                }
                                collide_h(m, omega, omega_u);
                                if (sr_on)
                                    store_scaled_sr<S>(dst, ai, m, rho0, sc, sr_key(sr_seed, x, y, z, nx, ny));
                                else
                                    store_scaled<S>(dst, ai, m, rho0, sc);
                            }
                        } else if (exp) {
                            // non-bulk node: hand its pulled populations to the node-list kernel
                            float fw[27];
                            gather_all<TY>(eup, efl, dn, col, p0, pp5, c6, fw);
                            float *pq = popbuf + (rq + __popc(bal & ((1u << tx) - 1u)));
#pragma unroll
                            for (int q = 0; q < 27; ++q) pq[(int64_t)q * n_pop] = fw[q];
                        }
                    }
                    if (k + 2 <= last) nb_arrive(3 + (k & 1), G::NTH);  // DONE(k)
                    soff += zst;
                }
                wq = wnew;
                rq = rnew;
                pp5 = p5;
                p5 = c5;
                p0 = c0;
                k3 = k3 == 2 ? 0 : k3 + 1;
                k4 = (k4 + 1) & 3;
            };
            for (int k = 0; k <= last; k += 2) {
                owner_plane(k, pa, pb, wqa, rqa, wqb);
                if (k + 1 <= last) owner_plane(k + 1, pb, pa, wqb, rqb, wqa);
            }
            if (diag) {
                dmD += (double)dm;
                deD += (double)de;
            }
        } else {
            auto rim_plane = [&](const int k, const Raw<S> &cur, Raw<S> &nxt) {
                if (k >= 4) nb_sync(3 + (k & 1), G::NTH);  // DONE(k-2): ring slots of plane k are free
                if (active) {
                    if (k < last) {
                        load_words<S>(src, loff, nxt);
                        loff += zst;
                        if (++zn == nz) {
                            zn = 0;
                            loff -= wrap;
                        }
                    }
                    arrive_rim<S, TY>(cur, rho0, sc, rside, up_base + k4 * G::PLANE, fl_base + k3 * G::PLANE,
                                      dn_base + (k & 1) * G::PLANE, ccol);
                }
                if (k >= 2) nb_arrive(1 + (k & 1), G::NTH);  // FULL(k)
                k3 = k3 == 2 ? 0 : k3 + 1;
                k4 = (k4 + 1) & 3;
            };
            for (int k = 0; k <= last; k += 2) {
                rim_plane(k, pa, pb);
                if (k + 1 <= last) rim_plane(k + 1, pb, pa);
            }
        }
        if (tid == 0) s_next = work ? (int)gridDim.x + atomicAdd(work, 1) : it + (int)gridDim.x;
        __syncthreads();  // the next item reuses the rings from slot 0
        it = s_next;
    }

    if (diag) {
        // deterministic block reduction of the owner threads' FP64 partials -> diag_part[blockIdx.x]
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            dmD += __shfl_down_sync(0xffffffffu, dmD, o);
            deD += __shfl_down_sync(0xffffffffu, deD, o);
        }
        if (tx == 0 && owner) {
            red[0][ty] = dmD;
            red[1][ty] = deD;
        }
        __syncthreads();
        if (tid == 0) {
            double s0 = 0.0, s1 = 0.0;
            for (int i = 0; i < TY; ++i) {
                s0 += red[0][i];
                s1 += red[1][i];
            }
            diag_part[2 * blockIdx.x + 0] = s0;
            diag_part[2 * blockIdx.x + 1] = s1;
        }
    }
}

__global__ void diag_finalize_kernel(const double *__restrict__ part, int n, double *__restrict__ out,
                                     int *__restrict__ error) {
    __shared__ double s[2][256];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        a += part[2 * i];
        b += part[2 * i + 1];
    }
    s[0][threadIdx.x] = a;
    s[1][threadIdx.x] = b;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            s[0][threadIdx.x] += s[0][threadIdx.x + o];
            s[1][threadIdx.x] += s[1][threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = s[0][0];
        out[1] = s[1][0];
        if (error && !(isfinite(s[0][0]) && isfinite(s[1][0]))) atomicOr(error, kErrorDiverged);
    }
}

// Opt the kernel into its dynamic shared memory once per device (the attribute belongs to the
// current device's context; never set inside a stream capture: batched launches are prepared
// before their graphs are captured).  Devices past the 64th are configured on every launch.
template <typename S, int TY, bool SP, bool BATCH, bool FULL = false>
cudaError_t configure_t() {
    static std::atomic<unsigned long long> configured{0ull};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = dev >= 0 && dev < 64 ? 1ull << dev : 0ull;
    if (bit && (configured.load(std::memory_order_acquire) & bit)) return cudaSuccess;
    e = cudaFuncSetAttribute(step_kernel<S, TY, SP, BATCH, FULL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             Geo<TY>::SMEM);
    if (e != cudaSuccess) return e;
    configured.fetch_or(bit, std::memory_order_acq_rel);
    return cudaSuccess;
}

template <typename S, int TY, bool SP, bool BATCH, bool FULL = false>
cudaError_t launch_t(const StepArgs *ga, const BatchArgs *ba, int parity, double *diag_part, int n_ctas,
                     cudaStream_t s) {
    const cudaError_t e = configure_t<S, TY, SP, BATCH, FULL>();
    if (e != cudaSuccess) return e;
    step_kernel<S, TY, SP, BATCH, FULL><<<n_ctas, Geo<TY>::NTH, Geo<TY>::SMEM, s>>>(ga, ba, parity, diag_part);
    return cudaGetLastError();
}

// `full`: whole tiles only; used by the single-case bulk variant (the other variants keep the
// ragged-edge predicates)
template <typename S, bool SP, bool BATCH>
cudaError_t launch_s(const StepArgs *ga, const BatchArgs *ba, int parity, double *diag_part, int n_ctas, int tile_y,
                     bool full, cudaStream_t s) {
    if constexpr (!SP && !BATCH) {
        if (full) {
            switch (tile_y) {
                case 4: return launch_t<S, 4, false, false, true>(ga, ba, parity, diag_part, n_ctas, s);
                case 8: return launch_t<S, 8, false, false, true>(ga, ba, parity, diag_part, n_ctas, s);
                case 16: return launch_t<S, 16, false, false, true>(ga, ba, parity, diag_part, n_ctas, s);
                default: return cudaErrorInvalidValue;
            }
        }
    }
    switch (tile_y) {
        case 4: return launch_t<S, 4, SP, BATCH>(ga, ba, parity, diag_part, n_ctas, s);
        case 8: return launch_t<S, 8, SP, BATCH>(ga, ba, parity, diag_part, n_ctas, s);
        case 16: return launch_t<S, 16, SP, BATCH>(ga, ba, parity, diag_part, n_ctas, s);
        default: return cudaErrorInvalidValue;
    }
}

template <typename S, int TY>
int occ_t() {
    int n = 0;
    cudaFuncSetAttribute(step_kernel<S, TY, true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         Geo<TY>::SMEM);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, step_kernel<S, TY, true, false, false>, Geo<TY>::NTH,
                                                      Geo<TY>::SMEM) !=
        cudaSuccess)
        return 0;
    return n;
}
template <typename S>
int occ_s(int ty) {
    switch (ty) {
        case 4: return occ_t<S, 4>();
        case 8: return occ_t<S, 8>();
        case 16: return occ_t<S, 16>();
        default: return 0;
    }
}

}  // namespace

cudaError_t launch_step(const StepLaunch &l, int storage, int tile_y, bool special, cudaStream_t s) {
    const StepArgs *ga = l.ga;
    switch (storage) {
        case MRLBM_STORAGE_F32:
            return special ? launch_s<float, true, false>(ga, nullptr, l.parity, l.diag_part, l.n_ctas, tile_y, false, s)
                           : launch_s<float, false, false>(ga, nullptr, l.parity, l.diag_part, l.n_ctas, tile_y,
                                                           l.full_tiles, s);
        case MRLBM_STORAGE_F16:
            return special ? launch_s<__half, true, false>(ga, nullptr, l.parity, l.diag_part, l.n_ctas, tile_y, false, s)
                           : launch_s<__half, false, false>(ga, nullptr, l.parity, l.diag_part, l.n_ctas, tile_y,
                                                            l.full_tiles, s);
        case MRLBM_STORAGE_BF16:
            return special ? launch_s<__nv_bfloat16, true, false>(ga, nullptr, l.parity, l.diag_part, l.n_ctas, tile_y,
                                                                  false, s)
                           : launch_s<__nv_bfloat16, false, false>(ga, nullptr, l.parity, l.diag_part, l.n_ctas,
                                                                   tile_y, l.full_tiles, s);
        case MRLBM_STORAGE_F16_U32:
            return special ? launch_s<HybridWord, true, false>(ga, nullptr, l.parity, l.diag_part, l.n_ctas, tile_y,
                                                                  false, s)
                           : launch_s<HybridWord, false, false>(ga, nullptr, l.parity, l.diag_part, l.n_ctas,
                                                                   tile_y, l.full_tiles, s);
        default: return cudaErrorInvalidValue;
    }
}

template <typename S, int TY>
cudaError_t prepare_ty() {
    const cudaError_t e = configure_t<S, TY, true, true>();
    return e != cudaSuccess ? e : configure_t<S, TY, false, true>();
}

template <typename S>
cudaError_t prepare_s(int tile_y) {
    switch (tile_y) {
        case 4: return prepare_ty<S, 4>();
        case 8: return prepare_ty<S, 8>();
        case 16: return prepare_ty<S, 16>();
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t prepare_step_batch(int storage, int tile_y) {
    switch (storage) {
        case MRLBM_STORAGE_F32: return prepare_s<float>(tile_y);
        case MRLBM_STORAGE_F16: return prepare_s<__half>(tile_y);
        case MRLBM_STORAGE_BF16: return prepare_s<__nv_bfloat16>(tile_y);
        case MRLBM_STORAGE_F16_U32: return prepare_s<HybridWord>(tile_y);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_step_batch(const BatchArgs *ba, int parity, int storage, int tile_y, bool special, int n_ctas,
                              cudaStream_t s) {
    switch (storage) {
        case MRLBM_STORAGE_F32:
            return special ? launch_s<float, true, true>(nullptr, ba, parity, nullptr, n_ctas, tile_y, false, s)
                           : launch_s<float, false, true>(nullptr, ba, parity, nullptr, n_ctas, tile_y, false, s);
        case MRLBM_STORAGE_F16:
            return special ? launch_s<__half, true, true>(nullptr, ba, parity, nullptr, n_ctas, tile_y, false, s)
                           : launch_s<__half, false, true>(nullptr, ba, parity, nullptr, n_ctas, tile_y, false, s);
        case MRLBM_STORAGE_BF16:
            return special ? launch_s<__nv_bfloat16, true, true>(nullptr, ba, parity, nullptr, n_ctas, tile_y, false, s)
                           : launch_s<__nv_bfloat16, false, true>(nullptr, ba, parity, nullptr, n_ctas, tile_y, false, s);
        case MRLBM_STORAGE_F16_U32:
            return special ? launch_s<HybridWord, true, true>(nullptr, ba, parity, nullptr, n_ctas, tile_y, false, s)
                           : launch_s<HybridWord, false, true>(nullptr, ba, parity, nullptr, n_ctas, tile_y, false, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_diag_finalize(const double *part, int n, double *out, int *error, cudaStream_t s) {
    diag_finalize_kernel<<<1, 256, 0, s>>>(part, n, out, error);
    return cudaGetLastError();
}

int step_kernel_smem_bytes(int tile_y) {
    switch (tile_y) {
        case 4: return Geo<4>::SMEM;
        case 8: return Geo<8>::SMEM;
        case 16: return Geo<16>::SMEM;
        default: return 0;
    }
}

int step_kernel_max_ctas_per_sm(int storage, int tile_y) {
    switch (storage) {
        case MRLBM_STORAGE_F32: return occ_s<float>(tile_y);
        case MRLBM_STORAGE_F16: return occ_s<__half>(tile_y);
        case MRLBM_STORAGE_BF16: return occ_s<__nv_bfloat16>(tile_y);
        case MRLBM_STORAGE_F16_U32: return occ_s<HybridWord>(tile_y);
        default: return 0;
    }
}

// ---- allocation-free periodic step --------------------------------------------------------
// For callers that cannot allocate device memory: the step kernel's own scratch (its argument
// block, work-item list, diagnostics partials and sums, error word) lives in this fixed array
// of the library's device image, kNoAllocScratchBytes = 64 KiB, laid out as in kernels.h.
// Every call shares it and it keeps the last call's contents; calls that overlap on the GPU
// (two streams, or two host threads) race on it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static_assert(sizeof(StepArgs) <= kNoAllocDiagOffset, "StepArgs outgrew its scratch slot");
static_assert(kNoAllocItemsOffset < kNoAllocScratchBytes, "scratch layout");

namespace {

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
// per device, set up on its first call: the scratch array's device address, the SM count and
// the resident step-kernel CTAs per SM
struct NoAllocDevice {
    void *scratch = nullptr;
    int n_sm = 0, per_sm = 0;
};
NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];

// Write the argument block, clear the error word and fill the work items (every xy tile of
// every z segment, segment-major) inside the scratch array: one launch, no host staging.
__global__ void noalloc_setup_kernel(const StepArgs a, unsigned char *scratch, int tiles, int n_items) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        *(StepArgs *)scratch = a;
        *(int *)(scratch + kNoAllocErrorOffset) = 0;
        *(int *)(scratch + kNoAllocWorkOffset) = 0;
    }
    int32_t *items = (int32_t *)(scratch + kNoAllocItemsOffset);
    for (int j = i; j < n_items; j += gridDim.x * blockDim.x) items[j] = (j % tiles) | ((j / tiles) << 20);
}

// Set-up of device `dev` (the current device), once: the scratch array's device address (in
// host code the array's name is only a host-side stand-in), its SM count and the step kernel's
// occupancy.  Host-side queries only; nothing is allocated.
cudaError_t noalloc_device(int dev, NoAllocDevice &out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if (!d.scratch) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        int n_sm = 0;
        if ((e = cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        d.n_sm = n_sm;
        d.per_sm = std::max(1, occ_s<float>(kNoAllocTileY));
        d.scratch = p;
    }
    out = d;
    return cudaSuccess;
}

int noalloc_cuda_fail(cudaError_t e, const char *what, std::string &err) {
    err = std::string("mrlbm_step_periodic_noalloc: ") + what + ": " + cudaGetErrorString(e);
    return e == cudaErrorNoKernelImageForDevice ? MRLBM_ERR_UNSUPPORTED : MRLBM_ERR_CUDA;
}

}  // namespace

int noalloc_periodic_step(const NoAllocStep &p, std::string &err) {
    const char *fn = "mrlbm_step_periodic_noalloc: ";
    // host-side checks first: nothing below runs for a rejected call
    if (!p.m_in || !p.m_out) {
        err = std::string(fn) + "null moment buffer";
        return MRLBM_ERR_INVALID_ARG;
    }
    if (p.nx <= 0 || p.ny <= 0 || p.nz <= 0 || p.nx % 8 || p.ny % 8 || p.nz % 4) {
        err = std::string(fn) + "grid must be positive multiples of 8 x 8 x 4";
        return MRLBM_ERR_INVALID_ARG;
    }
    if ((int64_t)p.nx * p.ny * p.nz >= (1LL << 31) * 8) {
        err = std::string(fn) + "grid too large";
        return MRLBM_ERR_INVALID_ARG;
    }
    if (!(p.omega > 0.f && p.omega < 2.f) || !(p.rho0 > 0.f) || !std::isfinite(p.rho0)) {
        err = std::string(fn) + "need 0 < omega < 2 and rho0 > 0";
        return MRLBM_ERR_INVALID_ARG;
    }
    if ((uintptr_t)p.m_in % 16 || (uintptr_t)p.m_out % 16) {
        err = std::string(fn) + "moment buffers must be 16-byte aligned";
        return MRLBM_ERR_INVALID_ARG;
    }
    const int64_t bytes = aos_elements(p.nx, p.ny, p.nz) * (int64_t)sizeof(float);
    const uintptr_t a = (uintptr_t)p.m_in, b = (uintptr_t)p.m_out;
    if ((a <= b ? b - a : a - b) < (uint64_t)bytes) {
        err = std::string(fn) + "input and output moment buffers overlap";
        return MRLBM_ERR_INVALID_ARG;
    }
    const int tiles_x = (p.nx + TILE_X - 1) / TILE_X, tiles_y = (p.ny + kNoAllocTileY - 1) / kNoAllocTileY;
    const int tiles = tiles_x * tiles_y;
    if (tiles > kNoAllocMaxItems) {
        err = std::string(fn) + "grid too large for the fixed 64 KiB scratch: " + std::to_string(tiles) +
              " xy tiles of 32 x 16 nodes, at most " + std::to_string(kNoAllocMaxItems);
        return MRLBM_ERR_INVALID_ARG;
    }

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_cuda_fail(e, "cudaGetDevice", err);
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        err = std::string(fn) + "device ordinal out of range";
        return MRLBM_ERR_UNSUPPORTED;
    }
    NoAllocDevice nd;
    if (!g_noalloc_dev[dev].scratch) {
        int major = 0, minor = 0;
        if ((e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev)) != cudaSuccess ||
            (e = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev)) != cudaSuccess)
            return noalloc_cuda_fail(e, "cudaDeviceGetAttribute", err);
        if (!(major == 10 && minor == 3)) {
            err = std::string(fn) + "libmrlbm is built for sm_103a (GB300) only";
            return MRLBM_ERR_UNSUPPORTED;
        }
    }
    if ((e = noalloc_device(dev, nd)) != cudaSuccess) return noalloc_cuda_fail(e, "device set-up", err);
    unsigned char *scratch = (unsigned char *)nd.scratch;

    // tiling: 32 x 16 columns; the longest z segment that still gives every resident CTA
    // several items, lengthened if the item list would not fit the scratch or the segment
    // number its 11-bit field of the work item (tile | segment << 20)
    const int resident = nd.per_sm * nd.n_sm;
    int lz = p.nz;
    while (lz > 16 && (int64_t)tiles * ((p.nz + lz - 1) / lz) < 4LL * resident) lz = (lz + 1) / 2;
    const int max_seg = std::min(kNoAllocMaxItems / tiles, 1 << 11);
    if ((p.nz + lz - 1) / lz > max_seg) lz = (p.nz + max_seg - 1) / max_seg;
    const int nseg = (p.nz + lz - 1) / lz;
    const int n_items = tiles * nseg;
    const int n_ctas = std::max(1, std::min(std::min(n_items, resident), kNoAllocMaxCtas));

    StepArgs sa;
    sa.m[0] = const_cast<float *>(p.m_in);
    sa.m[1] = p.m_out;
    sa.nxb = (p.nx + kXBlock - 1) / kXBlock;
    sa.items = (const int32_t *)(scratch + kNoAllocItemsOffset);
    sa.n_items = n_items;
    sa.nx = p.nx;
    sa.ny = p.ny;
    sa.nz = p.nz;
    sa.tiles_x = tiles_x;
    sa.tiles_y = tiles_y;
    sa.tile_y = kNoAllocTileY;
    sa.lz = lz;
    sa.omega = p.omega;
    sa.rho0 = p.rho0;
    for (int k = 0; k < 3; ++k) sa.sc.s[k] = sa.sc.is[k] = 1.f;
    sa.error = (int *)(scratch + kNoAllocErrorOffset);
    sa.work_counter = (int *)(scratch + kNoAllocWorkOffset);

    noalloc_setup_kernel<<<(n_items + 255) / 256, 256, 0, p.stream>>>(sa, scratch, tiles, n_items);
    if ((e = cudaGetLastError()) != cudaSuccess) return noalloc_cuda_fail(e, "set-up launch", err);
    StepLaunch L;
    L.ga = (const StepArgs *)scratch;
    L.parity = 0;
    L.n_ctas = n_ctas;
    double *part = (double *)(scratch + kNoAllocPartOffset);
    double *sums = (double *)(scratch + kNoAllocDiagOffset);
    if (p.diag_host) L.diag_part = part;
    if ((e = launch_t<float, kNoAllocTileY, false, false>(L.ga, nullptr, 0, L.diag_part, L.n_ctas, p.stream)) !=
        cudaSuccess)
        return noalloc_cuda_fail(e, "step launch", err);
    if (p.diag_host) {
        if ((e = launch_diag_finalize(part, n_ctas, sums, nullptr, p.stream)) != cudaSuccess)
            return noalloc_cuda_fail(e, "diagnostics launch", err);
        double v[2];
        if ((e = cudaMemcpyAsync(v, sums, sizeof(v), cudaMemcpyDeviceToHost, p.stream)) != cudaSuccess ||
            (e = cudaStreamSynchronize(p.stream)) != cudaSuccess)
            return noalloc_cuda_fail(e, "diagnostics read-back", err);
        p.diag_host[0] = (double)p.nx * p.ny * p.nz * p.rho0 + v[0];
        p.diag_host[1] = v[1];
        if (!std::isfinite(v[0]) || !std::isfinite(v[1])) {
            err = std::string(fn) + "mass / energy diagnostics are not finite";
            return MRLBM_ERR_DIVERGED;
        }
    }
    return MRLBM_OK;
}

}  // namespace mrlbm
