// Boundary and other non-bulk nodes: one thread per listed node, after the step kernel.
//
// The step kernel updates every plain bulk node in its fused pass, including plain fluid
// nodes whose only mark is the wall-stencil bit (it also writes their snapshot), and collides
// the solid nodes of updated blocks in place.  For every other node that carries a node word
// (domain faces / edges / corners, BCFLUID, BCSOLID, curved-wall nodes) it only exports the 27
// pulled populations to a list-ordered buffer; this kernel applies the node's closure,
// snapshots stencil nodes for the wall kernel, collides and stores.  Nodes of blocks the
// reference never updates (frozen) are in no list.  (The C_SOLID branch below is kept for a
// list that would carry solid nodes; the list built by the host holds none.)
//
// Reference (paths inside sakthi-lbm/MRLBM_3D_CUDA):
//   evaluate_bounday_moments dispatch   MRLBM_3D/src/solver/mlbm.cu:166-184
//   cylinder_boundary_moments / annulus_boundary_moments
//                                       MRLBM_3D/src/cases/cylinder/cylinder_kernels.cuh:32-65,
//                                       MRLBM_3D/src/cases/annulus/annulus_kernels.cuh:17-58
//   boundary_condition (faces, edges, corners), fluid_boundary_condition (BCFLUID),
//   bcsolid_boundary_condition (BCSOLID, z walls only)
//                                       MRLBM_3D/src/cases/cylinder/boundaries.cuh:8-1214
//   evaluate_incoming_moments_rotated   MRLBM_3D/src/boundary/curvedLBM.cu:5-59
//   moment_collision                    MRLBM_3D/src/solver/mlbm.cu:3-16
//   compute_force_mass_kernel (BCFLUID part)  MRLBM_3D/src/statistics/forces.cu:25-133
#include "mrlbm_internal.h"
#include "storage.cuh"

namespace mrlbm {
namespace {

// Density and velocity from a full set of 27 populations.
__device__ __forceinline__ Mom rho_u_of(const float *f) {
    float r = 0.f, jx = 0.f, jy = 0.f, jz = 0.f;
#pragma unroll
    for (int q = 0; q < 27; ++q) {
        r += f[q];
        jx += f[q] * (float)cxq(q);
        jy += f[q] * (float)cyq(q);
        jz += f[q] * (float)czq(q);
    }
    Mom m;
    const float inv = 1.0f / r;
    m.rho = r;
    m.ux = jx * inv;
    m.uy = jy * inv;
    m.uz = jz * inv;
    m.mxx = m.myy = m.mzz = m.mxy = m.mxz = m.myz = 0.f;
    return m;
}

// Post-stream density and velocity of node (x, y, z): its 27 populations pulled from the
// stored moments of the neighbours, on the grid that wraps in every axis.
template <typename S>
__device__ __noinline__ Mom pulled_rho_u(const StepArgs &a, const S *__restrict__ src, int x, int y, int z) {
    float f[27];
#pragma unroll 1
    for (int q = 0; q < 27; ++q) {
        const int xs = (x - cxq(q) + a.nx) % a.nx, ys = (y - cyq(q) + a.ny) % a.ny, zs = (z - czq(q) + a.nz) % a.nz;
        float raw[10], g[27];
        load_raw<S>(src, aos_at<S>(xs, ys, zs, a.nxb, a.ny), raw);
        rebuild<S>(raw, a.rho0, a.sc, g);
        f[q] = g[q];
    }
    return rho_u_of(f);
}

// Closure of one listed node from its pulled populations `fl`.  Returns 0 when the node is
// not stored here (wall nodes: the wall kernel finishes them), 1 to store the collided moments
// `m`, 2 to store them and count the node in the fluid diagnostics.
template <typename S>
__device__ __forceinline__ int special_node(const StepArgs &a, int parity, bool force, uint32_t w, const float *fl,
                                            int x, int y, int z, int slot, int x0, int y0, Mom &m) {
    const uint32_t cls = w & NW_CLASS_MASK;
    const S *__restrict__ src = (const S *)a.m[parity];
    bool wall_node = false;
    bool fluid = true;
    if (cls == C_BULK) {
        evaluate(fl, m);
    } else {
        const Mom prev = load_mom<S>(src, aos_at<S>(x, y, z, a.nxb, a.ny), a.rho0, a.sc);
        m = prev;  // nodes without a closure keep their pre-stream moments
        if (cls == C_SOLID) {
            fluid = false;
        } else if (cls == C_INNER || cls == C_OUTER) {
            const int wi = cls == C_INNER ? 0 : 1;
            const uint32_t bi = w >> NW_PAYLOAD_SHIFT;
            incoming_rotated(a.wall[wi].nx[bi], a.wall[wi].ny[bi], a.wall[wi].in_mask[bi], fl, m);
            wall_node = true;
            fluid = false;
        } else if (cls == C_BCFLUID_INNER || cls == C_BCFLUID_OUTER) {
            const uint32_t tag = (w >> NW_PAYLOAD_SHIFT) & 0xFFu;
            Mom o = prev;
            if (bcfluid_closure(tag, a.tag_in[tag], fl, a.bcf_strong, a.omega, o)) m = o;
        } else if (cls == C_BCSOLID_INNER || cls == C_BCSOLID_OUTER) {
            const uint32_t tag = (w >> NW_PAYLOAD_SHIFT) & 0xFFu;
            Mom o = prev;
            if (bcsolid_closure(tag, fl, a.omega, o)) m = o;
        } else {
            PlanarCtx c;
            c.omega = a.omega;
            c.u_max = a.u_max;
            c.rho0 = a.rho0;
            c.convective = a.convective;
            c.self_prev = prev;
            c.west_prev = prev;
            if (class_walls(cls) & 2u) {
                if (a.current_update) {
                    // NEUMANN_CURRENT_UPDATE (boundaries.cuh:96-161): post-stream rho, u of the
                    // x-1 neighbour and of the node itself instead of their stored moments
                    c.west_prev = pulled_rho_u<S>(a, src, x - 1, y, z);
                    c.self_prev = rho_u_of(fl);
                } else {
                    c.west_prev = load_mom<S>(src, aos_at<S>(x - 1, y, z, a.nxb, a.ny), a.rho0, a.sc);
                }
            }
            Mom o = prev;
            if (planar_closure(cls, fl, c, o)) m = o;
        }
    }
    if ((w & NW_STENCIL) && slot >= 0) {
        float *e = a.side + side_index(slot, x, y, z, x0, y0, a.nz, TILE_X, a.tile_y) * 16;
        e[0] = m.rho - a.rho0;
        e[1] = m.ux; e[2] = m.uy; e[3] = m.uz;
        e[4] = m.mxx; e[5] = m.myy; e[6] = m.mzz;
        e[7] = m.mxy; e[8] = m.mxz; e[9] = m.myz;
    }
    if (wall_node) return 0;
    const bool bcf = force && slot >= 0 && (cls == C_BCFLUID_INNER || cls == C_BCFLUID_OUTER);
    double fin[4] = {0.0, 0.0, 0.0, 0.0};
    const uint32_t tag = (w >> NW_PAYLOAD_SHIFT) & 0xFFu;
    if (bcf) masked_momentum(a.tag_in[tag], m, fin);
    collide(m, a.omega);
    if (bcf) {
        double fo[4];
        masked_momentum(a.tag_out[tag], m, fo);
        float *e = a.side + side_index(slot, x, y, z, x0, y0, a.nz, TILE_X, a.tile_y) * 16;
        e[10] = (float)(fin[0] - fo[0]);
        e[11] = (float)(fin[1] - fo[1]);
        e[12] = (float)(fin[2] - fo[2]);
        e[13] = (float)(fin[3] - fo[3]);
    }
    return fluid ? 2 : 1;
}

constexpr int kListThreads = 256;

// BATCH: each block serves the case named by its entry in BatchArgs::list_blocks.
template <typename S, bool BATCH>
__global__ void __launch_bounds__(kListThreads)
    special_list_kernel(const StepArgs *__restrict__ ga, const BatchArgs *__restrict__ ba, int parity, int force,
                        double *__restrict__ diag_part) {
    int b0 = blockIdx.x, nblk = gridDim.x;
    if constexpr (BATCH) {
        const int4 m = ba->list_blocks[blockIdx.x];
        ga = ba->cases[m.x];
        b0 = blockIdx.x - m.y;
        nblk = m.z;
    }
    const StepArgs &a = *ga;
    S *__restrict__ dst = (S *)a.m[parity ^ 1];
    const int n_pop = a.n_list_pop, n_all = a.n_list;
    double dm = 0.0, de = 0.0;
    for (int i = b0 * blockDim.x + threadIdx.x; i < n_all; i += nblk * blockDim.x) {
        const uint64_t p = a.list_xyz[i];
        const int x = (int)(p & 0x1FFFFFu), y = (int)((p >> 21) & 0x1FFFFFu), z = (int)(p >> 42);
        const uint32_t w = a.list_word[i];
        float f[27];
#pragma unroll
        for (int q = 0; q < 27; ++q) f[q] = a.popbuf[(int64_t)q * n_pop + i];
        const int tx = x / TILE_X, ty = y / a.tile_y;
        const int slot = a.tile_slot[ty * a.tiles_x + tx];
        Mom m;
        const int code = special_node<S>(a, parity, force != 0, w, f, x, y, z, slot, tx * TILE_X, ty * a.tile_y, m);
        if (code) {
            const int64_t ai = aos_at<S>(x, y, z, a.nxb, a.ny);
            if (kScaled<S> && a.sr_step)
                store_mom_sr<S>(dst, ai, m, a.rho0, a.sc, sr_key(sr_step_seed(*a.sr_step), x, y, z, a.nx, a.ny));
            else
                store_mom<S>(dst, ai, m, a.rho0, a.sc);
        }
        if (code == 2 && diag_part) {
            dm += (double)(m.rho - a.rho0);
            de += 0.5 * (double)(m.ux * m.ux + m.uy * m.uy + m.uz * m.uz);
        }
    }
    if (diag_part) {
        // fixed-order block reduction -> diag_part[blockIdx.x]
        __shared__ double red[2][kListThreads / 32];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            dm += __shfl_down_sync(0xffffffffu, dm, o);
            de += __shfl_down_sync(0xffffffffu, de, o);
        }
        if ((threadIdx.x & 31) == 0) {
            red[0][threadIdx.x >> 5] = dm;
            red[1][threadIdx.x >> 5] = de;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double s0 = 0.0, s1 = 0.0;
            for (int k = 0; k < kListThreads / 32; ++k) {
                s0 += red[0][k];
                s1 += red[1][k];
            }
            diag_part[2 * blockIdx.x + 0] = s0;
            diag_part[2 * blockIdx.x + 1] = s1;
        }
    }
}

}  // namespace

int special_list_blocks(int n_list) {
    const int b = (n_list + kListThreads - 1) / kListThreads;
    return b < 1 ? 1 : (b > 2048 ? 2048 : b);
}

cudaError_t launch_special_list(const StepLaunch &l, int storage, int n_blocks, double *diag_part, cudaStream_t s) {
    const int f = l.force != nullptr;
    switch (storage) {
        case MRLBM_STORAGE_F32:
            special_list_kernel<float, false><<<n_blocks, kListThreads, 0, s>>>(l.ga, nullptr, l.parity, f, diag_part);
            break;
        case MRLBM_STORAGE_F16:
            special_list_kernel<__half, false><<<n_blocks, kListThreads, 0, s>>>(l.ga, nullptr, l.parity, f, diag_part);
            break;
        case MRLBM_STORAGE_BF16:
            special_list_kernel<__nv_bfloat16, false>
                <<<n_blocks, kListThreads, 0, s>>>(l.ga, nullptr, l.parity, f, diag_part);
            break;
        case MRLBM_STORAGE_F16_U32:
            special_list_kernel<HybridWord, false>
                <<<n_blocks, kListThreads, 0, s>>>(l.ga, nullptr, l.parity, f, diag_part);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_special_list_batch(const BatchArgs *ba, int parity, int force, int storage, int n_blocks,
                                      cudaStream_t s) {
    if (n_blocks <= 0) return cudaSuccess;
    switch (storage) {
        case MRLBM_STORAGE_F32:
            special_list_kernel<float, true><<<n_blocks, kListThreads, 0, s>>>(nullptr, ba, parity, force, nullptr);
            break;
        case MRLBM_STORAGE_F16:
            special_list_kernel<__half, true><<<n_blocks, kListThreads, 0, s>>>(nullptr, ba, parity, force, nullptr);
            break;
        case MRLBM_STORAGE_BF16:
            special_list_kernel<__nv_bfloat16, true>
                <<<n_blocks, kListThreads, 0, s>>>(nullptr, ba, parity, force, nullptr);
            break;
        case MRLBM_STORAGE_F16_U32:
            special_list_kernel<HybridWord, true>
                <<<n_blocks, kListThreads, 0, s>>>(nullptr, ba, parity, force, nullptr);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace mrlbm
