// Curved-wall boundary nodes: interpolated, rotated, extrapolated moment closure, then
// collision, plus the FP64 momentum-exchange force / torque sums.
//
// Reference (paths inside sakthi-lbm/MRLBM_3D_CUDA):
//   apply_bc_cylinder / apply_bc_annulus      MRLBM_3D/src/cases/cylinder/cylinder_kernels.cu:68-128,
//                                             MRLBM_3D/src/cases/annulus/annulus_kernels.cu:75-139
//   curved_boundary_condition_rotated         MRLBM_3D/src/boundary/curvedLBM.cu:61-132
//   bilinear_interpolation / extrapolation_quadratic / rotate_velocity_moments
//                                             MRLBM_3D/src/boundary/extrapolation_utils.cuh:5-107
//   numerical_solution_rhoeq_rotated / _strong_rotated
//                                             MRLBM_3D/src/boundary/numerical_solution.cu:4-279
//   compute_force_mass_kernel                 MRLBM_3D/src/statistics/forces.cu:25-133
// The reference runs this closure in its own kernel between the streaming and collision
// kernels and interpolates from the moment arrays while it overwrites boundary nodes in the
// same launch.  Here the step kernel leaves every stencil node's post-stream moments in a
// side buffer, this kernel reads only that snapshot (no read/write race) and writes the
// collided moments of the wall nodes straight into the next ping-pong buffer.
#include "mrlbm_internal.h"
#include "storage.cuh"

namespace mrlbm {
namespace {

struct VM {
    float ux, uy, uz, mxx, myy, mzz, mxy, mxz, myz;
};

__device__ __forceinline__ const float *side_entry(const StepArgs &a, int x, int y, int z) {
    if (x < 0 || x >= a.nx || y < 0 || y >= a.ny) return nullptr;
    const int tx = x / TILE_X, ty = y / a.tile_y;
    const int slot = a.tile_slot[ty * a.tiles_x + tx];
    if (slot < 0) return nullptr;
    return a.side + side_index(slot, x, y, z, tx * TILE_X, ty * a.tile_y, a.nz, TILE_X, a.tile_y) * 16;
}

// Bilinear interpolation of the 9 velocity / second-moment fields in the plane z, then
// rotation into the wall frame (cos = nx, sin = ny).
__device__ __forceinline__ bool interp_rotate(const StepArgs &a, float nx, float ny, float px, float py, int z,
                                              VM &vm) {
    const int x0 = (int)floorf(px), y0 = (int)floorf(py);
    const float xd = px - (float)x0, yd = py - (float)y0;
    const float *q00 = side_entry(a, x0, y0, z), *q10 = side_entry(a, x0 + 1, y0, z);
    const float *q01 = side_entry(a, x0, y0 + 1, z), *q11 = side_entry(a, x0 + 1, y0 + 1, z);
    if (!q00 || !q10 || !q01 || !q11) return false;
    float v[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const float r0 = (1.0f - xd) * q00[k + 1] + xd * q10[k + 1];
        const float r1 = (1.0f - xd) * q01[k + 1] + xd * q11[k + 1];
        v[k] = (1.0f - yd) * r0 + yd * r1;
    }
    const float ux = v[0], uy = v[1], uz = v[2], mxx = v[3], myy = v[4], mzz = v[5], mxy = v[6], mxz = v[7],
                myz = v[8];
    const float c = nx, s = ny;
    const float s2 = 2.0f * s * c, c2 = c * c - s * s;
    vm.ux = ux * c + uy * s;
    vm.uy = -ux * s + uy * c;
    vm.uz = uz;
    vm.mxx = mxx * c * c + myy * s * s + mxy * s2;
    vm.myy = mxx * s * s + myy * c * c - mxy * s2;
    vm.mzz = mzz;
    vm.mxy = mxy * c2 + 0.5f * (myy - mxx) * s2;
    vm.mxz = mxz * c + myz * s;
    vm.myz = myz * c - mxz * s;
    return true;
}

// Three-point extrapolation to the node at distance delta inside the wall from the wall
// value and the two fluid points at 1 and 2 lattice units (extrapolation_utils.cuh:49-61).
__device__ __forceinline__ float extrapolate(float d, float vw, float v1, float v2) {
    const float d2 = d * d;
    const float c1 = 1.0f - 0.5f * d2 + 1.5f * d;
    const float c2 = d2 - 2.0f * d;
    const float c3 = -0.5f * (d2 - d);
    return c1 * vw + c2 * v1 + c3 * v2;
}

// Moment closure in the rotated frame: the wall-parallel moments come from the
// extrapolation, m'_xy, m'_xz and rho from the incoming-population balance (a 2x2 solve).
__device__ void closure_rotated(const StepArgs &a, float c, float s, uint32_t inm, uint32_t outm, const VM &e, Mom &m) {
    const float s2 = 2.0f * s * c, c2 = c * c - s * s;
    constexpr float cbf = 4.5f;  // 0.5 * 3 * 3
    float A = 0.f, E = 0.f, Dxy = 0.f, Dxz = 0.f;
    float B11 = 0.f, B22 = 0.f, B33 = 0.f, B12 = 0.f, B13 = 0.f, B23 = 0.f;
    float F11y = 0.f, F22y = 0.f, F33y = 0.f, F12y = 0.f, F13y = 0.f, F23y = 0.f;
    float F11z = 0.f, F22z = 0.f, F33z = 0.f, F12z = 0.f, F13z = 0.f, F23z = 0.f;
    const bool strong = a.wall_strong != 0;
#pragma unroll
    for (int q = 0; q < 27; ++q) {
        const float cx = (float)cxq(q), cy = (float)cyq(q), cz = (float)czq(q);
        const float cxp = cx * c + cy * s;
        const float cyp = -cx * s + cy * c;
        const float czp = cz;
        const float hxx = cxp * cxp - kCs2, hyy = cyp * cyp - kCs2, hzz = czp * czp - kCs2;
        const float hxy = cxp * cyp, hxz = cxp * czp, hyz = cyp * czp;
        const float wq = weight(q);
        const float cf = cbf * wq;
        const float Ai = wq * (1.0f + 3.0f * (e.ux * cxp + e.uy * cyp + e.uz * czp));
        const float Ei = Ai + cf * (e.ux * e.ux * hxx + e.uy * e.uy * hyy + e.uz * e.uz * hzz + 2.0f * e.ux * e.uy * hxy +
                                    2.0f * e.ux * e.uz * hxz + 2.0f * e.uy * e.uz * hyz);
        if (strong ? (outm & (1u << q)) != 0 : false) {
            A += Ai;
            E += Ei;
            B11 += cf * hxx; B22 += cf * hyy; B33 += cf * hzz;
            B12 += cf * hxy; B13 += cf * hxz; B23 += cf * hyz;
        }
        if (inm & (1u << q)) {
            if (!strong) E += Ei;
            Dxy += Ai * hxy;
            Dxz += Ai * hxz;
            F11y += (cf * hxx) * hxy; F22y += (cf * hyy) * hxy; F33y += (cf * hzz) * hxy;
            F12y += (cf * hxy) * hxy; F13y += (cf * hxz) * hxy; F23y += (cf * hyz) * hxy;
            F11z += (cf * hxx) * hxz; F22z += (cf * hyy) * hxz; F33z += (cf * hzz) * hxz;
            F12z += (cf * hxy) * hxz; F13z += (cf * hxz) * hxz; F23z += (cf * hyz) * hxz;
        }
    }
    const float rhoI = m.rho, mxyI = m.mxy, mxzI = m.mxz;
    float G = E;
    if (strong) {
        const float om1 = 1.0f - a.omega;
        G = om1 * A + a.omega * E;
        const float ty = om1 * mxyI, tz = om1 * mxzI;
        F11y -= ty * B11; F22y -= ty * B22; F33y -= ty * B33; F12y -= ty * B12; F13y -= ty * B13; F23y -= ty * B23;
        F11z -= tz * B11; F22z -= tz * B22; F33z -= tz * B33; F12z -= tz * B12; F13z -= tz * B13; F23z -= tz * B23;
    }
    const float Rxy = G * mxyI - Dxy, Rxz = G * mxzI - Dxz;
    const float a1 = 2.0f * F12y, b1 = 2.0f * F13y;
    const float c1 = Rxy - e.mxx * F11y - e.myy * F22y - e.mzz * F33y - 2.0f * e.myz * F23y;
    const float a2 = 2.0f * F12z, b2 = 2.0f * F13z;
    const float c2v = Rxz - e.mxx * F11z - e.myy * F22z - e.mzz * F33z - 2.0f * e.myz * F23z;
    const float inv = 1.0f / (a2 * b1 - a1 * b2);
    const float mxyp = (b1 * c2v - b2 * c1) * inv;
    const float mxzp = (a2 * c1 - a1 * c2v) * inv;
    m.ux = e.ux * c - e.uy * s;
    m.uy = e.ux * s + e.uy * c;
    m.uz = e.uz;
    m.mxx = e.mxx * c * c + e.myy * s * s - mxyp * s2;
    m.myy = e.mxx * s * s + e.myy * c * c + mxyp * s2;
    m.mzz = e.mzz;
    m.mxy = (e.mxx - e.myy) * 0.5f * s2 + mxyp * c2;
    m.mxz = mxzp * c - e.myz * s;
    m.myz = mxzp * s + e.myz * c;
    if (strong) {
        const float om1 = 1.0f - a.omega;
        const float den = G + om1 * (e.mxx * B11 + e.myy * B22 + e.mzz * B33 + 2.0f * mxyp * B12 + 2.0f * mxzp * B13 +
                                     2.0f * e.myz * B23);
        m.rho = rhoI / den;
    } else {
        m.rho = rhoI / E;
    }
}

// BATCH: each block serves the case named by its entry in BatchArgs::wall_blocks; the force
// sums of a sampled step go to that case's ring slot BatchArgs::force_slot.
template <typename S, bool BATCH>
__global__ void __launch_bounds__(128)
    wall_kernel(const StepArgs *__restrict__ ga, const BatchArgs *__restrict__ ba, int parity, double *force) {
    int b0 = blockIdx.x;
    if constexpr (BATCH) {
        const int4 m = ba->wall_blocks[blockIdx.x];
        ga = ba->cases[m.x];
        b0 = blockIdx.x - m.y;
        force = force ? ba->force_ring[m.x] + (int64_t)(*ba->force_slot) * 10 : nullptr;
    }
    const StepArgs &a = *ga;
    const int nb0 = a.wall[0].nb, nb1 = a.wall[1].nb;
    const int nbf0 = force ? a.wall[0].nbf : 0, nbf1 = force ? a.wall[1].nbf : 0;
    const int n_total = nb0 + nb1 + nbf0 + nbf1;
    const int i = b0 * blockDim.x + threadIdx.x;
    const int64_t plane = (int64_t)a.nx * a.ny;
    double acc[2][5] = {{0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}};
    if (i < nb0 + nb1) {
        const int wi = i < nb0 ? 0 : 1;
        const int bi = i < nb0 ? i : i - nb0;
        const WallArgs &W = a.wall[wi];
        const int64_t node = W.list[bi];
        const int x = (int)(node % a.nx), y = (int)((node / a.nx) % a.ny), z = (int)(node / plane);
        const float *e0 = side_entry(a, x, y, z);
        if (!e0) {
            atomicOr(a.error, 1);
        } else {
            Mom m;
            m.rho = a.rho0 + e0[0];
            m.ux = e0[1]; m.uy = e0[2]; m.uz = e0[3];
            m.mxx = e0[4]; m.myy = e0[5]; m.mzz = e0[6];
            m.mxy = e0[7]; m.mxz = e0[8]; m.myz = e0[9];
            const float nx = W.nx[bi], ny = W.ny[bi], delta = W.delta[bi];
            const uint32_t inm = W.in_mask[bi], outm = W.out_mask[bi];
            const float xw = a.xc + W.r_wall * nx, yw = a.yc + W.r_wall * ny;
            const float x1 = xw + W.dir * nx, y1 = yw + W.dir * ny;
            const float x2 = xw + W.dir * 2.0f * nx, y2 = yw + W.dir * 2.0f * ny;
            VM v1, v2;
            const bool ok = interp_rotate(a, nx, ny, x1, y1, z, v1) && interp_rotate(a, nx, ny, x2, y2, z, v2);
            if (!ok) {
                atomicOr(a.error, 2);
            } else {
                const float uw = W.u_wall[0], vw = W.u_wall[1], ww = W.u_wall[2];
                VM ex;
                ex.ux = extrapolate(delta, uw, v1.ux, v2.ux);
                ex.uy = extrapolate(delta, vw, v1.uy, v2.uy);
                ex.uz = extrapolate(delta, ww, v1.uz, v2.uz);
                ex.mxx = extrapolate(delta, uw * uw, v1.mxx, v2.mxx);
                ex.myy = extrapolate(delta, vw * vw, v1.myy, v2.myy);
                ex.mzz = extrapolate(delta, ww * ww, v1.mzz, v2.mzz);
                ex.myz = extrapolate(delta, vw * ww, v1.myz, v2.myz);
                ex.mxy = ex.mxz = 0.f;
                closure_rotated(a, nx, ny, inm, outm, ex, m);
                double fin[4] = {0.0, 0.0, 0.0, 0.0}, fo[4];
                if (force) masked_momentum(inm, m, fin);
                collide(m, a.omega);
                const int64_t ai = aos_at<S>(x, y, z, a.nxb, a.ny);
                if (kScaled<S> && a.sr_step)
                    store_mom_sr<S>((S *)a.m[parity ^ 1], ai, m, a.rho0, a.sc,
                                    sr_key(sr_step_seed(*a.sr_step), x, y, z, a.nx, a.ny));
                else
                    store_mom<S>((S *)a.m[parity ^ 1], ai, m, a.rho0, a.sc);
                if (force) {
                    masked_momentum(outm, m, fo);
                    const double fx = fin[0] - fo[0], fy = fin[1] - fo[1];
                    acc[wi][0] = fx;
                    acc[wi][1] = fy;
                    acc[wi][2] = fin[2] - fo[2];
                    acc[wi][3] = fin[3] - fo[3];
                    acc[wi][4] = ((double)x - a.xc) * fy - ((double)y - a.yc) * fx;
                }
            }
        }
    } else if (i < n_total) {
        const int j = i - nb0 - nb1;
        const int wi = j < nbf0 ? 0 : 1;
        const int64_t node = a.wall[wi].fluid_list[j < nbf0 ? j : j - nbf0];
        const int x = (int)(node % a.nx), y = (int)((node / a.nx) % a.ny), z = (int)(node / plane);
        const float *e = side_entry(a, x, y, z);
        if (!e) {
            atomicOr(a.error, 4);
        } else {
            const double fx = e[10], fy = e[11];
            acc[wi][0] = fx;
            acc[wi][1] = fy;
            acc[wi][2] = e[12];
            acc[wi][3] = e[13];
            acc[wi][4] = ((double)x - a.xc) * fy - ((double)y - a.yc) * fx;
        }
    }
    if (!force) return;
    __shared__ double red[10][128];
#pragma unroll
    for (int k = 0; k < 10; ++k) red[k][threadIdx.x] = acc[k / 5][k % 5];
    __syncthreads();
    for (int o = 64; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
#pragma unroll
            for (int k = 0; k < 10; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x < 10) atomicAdd(force + threadIdx.x, red[threadIdx.x][0]);
}

}  // namespace

cudaError_t launch_wall(const StepLaunch &l, int storage, int n_total, cudaStream_t s) {
    if (n_total <= 0) return cudaSuccess;
    const int blocks = (n_total + 127) / 128;
    switch (storage) {
        case MRLBM_STORAGE_F32: wall_kernel<float, false><<<blocks, 128, 0, s>>>(l.ga, nullptr, l.parity, l.force); break;
        case MRLBM_STORAGE_F16: wall_kernel<__half, false><<<blocks, 128, 0, s>>>(l.ga, nullptr, l.parity, l.force); break;
        case MRLBM_STORAGE_BF16:
            wall_kernel<__nv_bfloat16, false><<<blocks, 128, 0, s>>>(l.ga, nullptr, l.parity, l.force);
            break;
        case MRLBM_STORAGE_F16_U32:
            wall_kernel<HybridWord, false><<<blocks, 128, 0, s>>>(l.ga, nullptr, l.parity, l.force);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_wall_batch(const BatchArgs *ba, int parity, int force, int storage, int n_blocks, cudaStream_t s) {
    if (n_blocks <= 0) return cudaSuccess;
    // any non-null pointer switches force accumulation on; the kernel takes the case's slot
    double *f = force ? reinterpret_cast<double *>(1) : nullptr;
    switch (storage) {
        case MRLBM_STORAGE_F32: wall_kernel<float, true><<<n_blocks, 128, 0, s>>>(nullptr, ba, parity, f); break;
        case MRLBM_STORAGE_F16: wall_kernel<__half, true><<<n_blocks, 128, 0, s>>>(nullptr, ba, parity, f); break;
        case MRLBM_STORAGE_BF16:
            wall_kernel<__nv_bfloat16, true><<<n_blocks, 128, 0, s>>>(nullptr, ba, parity, f);
            break;
        case MRLBM_STORAGE_F16_U32:
            wall_kernel<HybridWord, true><<<n_blocks, 128, 0, s>>>(nullptr, ba, parity, f);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

namespace {
__global__ void batch_force_begin_kernel(double *const *ring, int n_cases, int slot, int *d_slot) {
    for (int i = threadIdx.x; i < n_cases * 10; i += blockDim.x) ring[i / 10][(int64_t)slot * 10 + i % 10] = 0.0;
    if (threadIdx.x == 0) *d_slot = slot;
}
}  // namespace

cudaError_t launch_batch_force_begin(double *const *ring, int n_cases, int slot, int *d_slot, cudaStream_t s) {
    batch_force_begin_kernel<<<1, 256, 0, s>>>(ring, n_cases, slot, d_slot);
    return cudaGetLastError();
}

}  // namespace mrlbm
