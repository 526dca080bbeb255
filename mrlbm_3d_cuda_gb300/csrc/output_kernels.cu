// Device side of the reference-format outputs: the face-population halo of a restart.bin
// checkpoint and the time-averaged surface pressure of pressure.dat.
//
// Reference (paths inside sakthi-lbm/MRLBM_3D_CUDA):
//   pop_save_to_halo / idxPopX / idxPopY / idxPopZ   MRLBM_3D/src/core/D3Q27/halo_interface.cuh:109-201,
//                                                    MRLBM_3D/src/core/index.cuh:42-79
//   write_checkpoint                                 MRLBM_3D/src/restart/restart_io.cu:3-76
//   compute_surface_pressure                         MRLBM_3D/src/cases/cylinder/cylinder_kernels.cu:238-283
//   bilinear_interpolation, surface_pressure_extrapolation
//                                                    MRLBM_3D/src/boundary/extrapolation_utils.cuh:5-40,109-154
//   inlet_avg_density / compute_inlet_average_density, the running mean of cylinder_post_process
//                                                    MRLBM_3D/src/cases/cylinder/cylinder_kernels.cu:147-175,285-338
// The reference keeps the populations that cross its 8 x 8 x 4 block faces in six arrays
// between its two kernels; this solver has no such arrays (populations are rebuilt from the
// post-collision moments inside the fused step), so a checkpoint rebuilds them the same way:
// face populations = reconstruction of the node's stored moments.
#include "mrlbm_internal.h"
#include "storage.cuh"

namespace mrlbm {
namespace {

// Reference block of the halo layout.
constexpr int kBX = 8, kBY = 8, kBZ = 4, kQF = 9;

// j-th direction (ascending q) whose velocity component along `axis` equals `sign`: the nine
// populations that leave a block through that face.
__host__ __device__ constexpr int face_pop(int axis, int sign, int j) {
    for (int q = 1; q < 27; ++q) {
        const int c = axis == 0 ? cxq(q) : (axis == 1 ? cyq(q) : czq(q));
        if (c == sign && j-- == 0) return q;
    }
    return -1;
}
static_assert(face_pop(0, -1, 0) == 2 && face_pop(0, 1, 8) == 26 && face_pop(2, 1, 8) == 25,
              "face populations follow the reference's D3Q27 order");

template <typename S>
__global__ void halo_export_kernel(const StepArgs *__restrict__ ga, int parity, float *__restrict__ west,
                                   float *__restrict__ east, float *__restrict__ south, float *__restrict__ north,
                                   float *__restrict__ back, float *__restrict__ front) {
    const StepArgs &a = *ga;
    const int64_t n = (int64_t)a.nx * a.ny * a.nz;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % a.nx), y = (int)((i / a.nx) % a.ny), z = (int)(i / ((int64_t)a.nx * a.ny));
    const int tx = x % kBX, ty = y % kBY, tz = z % kBZ;
    const bool wx = tx == 0, ex = tx == kBX - 1, sy = ty == 0, ny_ = ty == kBY - 1, bz = tz == 0, fz = tz == kBZ - 1;
    if (!(wx || ex || sy || ny_ || bz || fz)) return;
    const int64_t gx = a.nx / kBX, gy = a.ny / kBY;
    const int64_t block = x / kBX + gx * (y / kBY + gy * (z / kBZ));
    float raw[10], f[27];
    load_raw<S>((const S *)a.m[parity], aos_at<S>(x, y, z, a.nxb, a.ny), raw);
    rebuild<S>(raw, a.rho0, a.sc, f);
#pragma unroll
    for (int j = 0; j < kQF; ++j) {
        const int64_t px = ty + kBY * (tz + kBZ * (j + kQF * block));
        const int64_t py = tx + kBX * (tz + kBZ * (j + kQF * block));
        const int64_t pz = tx + kBX * (ty + kBY * (j + kQF * block));
        if (wx) west[px] = f[face_pop(0, -1, j)];
        if (ex) east[px] = f[face_pop(0, 1, j)];
        if (sy) south[py] = f[face_pop(1, -1, j)];
        if (ny_) north[py] = f[face_pop(1, 1, j)];
        if (bz) back[pz] = f[face_pop(2, -1, j)];
        if (fz) front[pz] = f[face_pop(2, 1, j)];
    }
}

// Density deviation at (x, y, z) of the stored moments.
template <typename S>
__device__ __forceinline__ float rho_dev(const StepArgs &a, const S *m, int x, int y, int z) {
    const float v = load_field<S>(m, aos_at<S>(x, y, z, a.nxb, a.ny), 0);
    return std::is_same<S, float>::value ? v : v * a.sc.is[0];
}

// Pressure at the wall point from three probes along the normal: the quadratic in r through
// (r_k, cs2 rho_k), k = 1..3, evaluated at r_w.
__device__ __forceinline__ float wall_pressure(float xc, float yc, float xw, float yw, const float px[3],
                                               const float py[3], const float rho[3]) {
    const float rw = sqrtf((xw - xc) * (xw - xc) + (yw - yc) * (yw - yc));
    float r[3], p[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        r[k] = sqrtf((px[k] - xc) * (px[k] - xc) + (py[k] - yc) * (py[k] - yc));
        p[k] = rho[k] * kCs2;
    }
    const float den = (r[0] - r[1]) * (r[0] - r[2]) * (r[1] - r[2]);
    const float a0 = (r[0] * r[2] * p[1] * (r[2] - r[0]) + (r[1] * r[1]) * (r[2] * p[0] - r[0] * p[2]) +
                      r[1] * ((r[0] * r[0]) * p[2] - (r[2] * r[2]) * p[0])) / den;
    const float a1 = ((r[2] * r[2]) * (p[0] - p[1]) + (r[0] * r[0]) * (p[1] - p[2]) + (r[1] * r[1]) * (p[2] - p[0])) / den;
    const float a2 = (r[2] * (p[1] - p[0]) + r[1] * (p[0] - p[2]) + r[0] * (p[2] - p[1])) / den;
    return a0 + a1 * rw + a2 * (rw * rw);
}

template <typename S>
__global__ void surface_pressure_kernel(const StepArgs *__restrict__ ga, int buf, int wall, double *__restrict__ avg,
                                        int n_avg) {
    const StepArgs &a = *ga;
    const WallArgs &W = a.wall[wall];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= W.nb) return;
    const int64_t node = W.list[i];
    const int64_t plane = (int64_t)a.nx * a.ny;
    const int z = (int)(node / plane);
    const float nx = W.nx[i], ny = W.ny[i];
    const float xw = a.xc + W.r_wall * nx, yw = a.yc + W.r_wall * ny;
    const S *m = (const S *)a.m[buf];
    float px[3], py[3], rho[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        px[k] = xw + W.dir * (float)(k + 1) * nx;
        py[k] = yw + W.dir * (float)(k + 1) * ny;
        const int x0 = (int)floorf(px[k]), y0 = (int)floorf(py[k]);
        const float xd = px[k] - (float)x0, yd = py[k] - (float)y0;
        const bool in = x0 >= 0 && y0 >= 0 && x0 + 1 < a.nx && y0 + 1 < a.ny;
        if (!in) {
            atomicOr(a.error, 8);
            return;
        }
        const float q00 = rho_dev<S>(a, m, x0, y0, z), q10 = rho_dev<S>(a, m, x0 + 1, y0, z);
        const float q01 = rho_dev<S>(a, m, x0, y0 + 1, z), q11 = rho_dev<S>(a, m, x0 + 1, y0 + 1, z);
        const float r0 = (1.0f - xd) * q00 + xd * q10, r1 = (1.0f - xd) * q01 + xd * q11;
        rho[k] = a.rho0 + ((1.0f - yd) * r0 + yd * r1);
    }
    const double ps = (double)wall_pressure(a.xc, a.yc, xw, yw, px, py, rho);
    avg[i] += (ps - avg[i]) / (double)n_avg;  // running mean over the sampled steps
}

// Mean density of the x = 0 face (ny * nz nodes) and its running mean over the statistics
// window.  One block, FP64 sums in a fixed order (the reference sums in FP32 with atomics).
// state[0] is the running mean; slot entry = (this sample, the mean of the earlier samples):
// the reference writes its inlet_density.dat line before it updates the mean.
constexpr int kInletThreads = 512;

template <typename S>
__global__ void __launch_bounds__(kInletThreads)
    inlet_density_kernel(const StepArgs *__restrict__ ga, int buf, double *__restrict__ state, int slot, int n_avg) {
    const StepArgs &a = *ga;
    const S *m = (const S *)a.m[buf];
    const int n = a.ny * a.nz;
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += kInletThreads) {
        const int y = i % a.ny, z = i / a.ny;
        s += (double)(a.rho0 + rho_dev<S>(a, m, 0, y, z));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ double part[kInletThreads / 32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kInletThreads / 32; ++w) t += part[w];
        const double in = t / (double)n;
        double *e = state + 1 + 2 * (int64_t)slot;
        e[0] = in;
        e[1] = state[0];
        state[0] += (in - state[0]) / (double)n_avg;
    }
}

}  // namespace

int64_t halo_face_floats(int nx, int ny, int nz, int axis) {
    const int64_t blocks = (int64_t)(nx / kBX) * (ny / kBY) * (nz / kBZ);
    const int64_t face = axis == 0 ? kBY * kBZ : (axis == 1 ? kBX * kBZ : kBX * kBY);
    return face * blocks * kQF;
}

cudaError_t launch_halo_export(const StepArgs *ga, int parity, int storage, int64_t n, float *const faces[6],
                               cudaStream_t s) {
    const unsigned blocks = (unsigned)((n + 255) / 256);
    switch (storage) {
        case MRLBM_STORAGE_F32:
            halo_export_kernel<float><<<blocks, 256, 0, s>>>(ga, parity, faces[0], faces[1], faces[2], faces[3],
                                                             faces[4], faces[5]);
            break;
        case MRLBM_STORAGE_F16:
            halo_export_kernel<__half><<<blocks, 256, 0, s>>>(ga, parity, faces[0], faces[1], faces[2], faces[3],
                                                              faces[4], faces[5]);
            break;
        case MRLBM_STORAGE_BF16:
            halo_export_kernel<__nv_bfloat16><<<blocks, 256, 0, s>>>(ga, parity, faces[0], faces[1], faces[2],
                                                                     faces[3], faces[4], faces[5]);
            break;
        case MRLBM_STORAGE_F16_U32:
            halo_export_kernel<HybridWord><<<blocks, 256, 0, s>>>(ga, parity, faces[0], faces[1], faces[2],
                                                                     faces[3], faces[4], faces[5]);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_inlet_density(const StepArgs *ga, int buf, int storage, double *state, int slot, int n_avg,
                                 cudaStream_t s) {
    switch (storage) {
        case MRLBM_STORAGE_F32: inlet_density_kernel<float><<<1, kInletThreads, 0, s>>>(ga, buf, state, slot, n_avg); break;
        case MRLBM_STORAGE_F16:
            inlet_density_kernel<__half><<<1, kInletThreads, 0, s>>>(ga, buf, state, slot, n_avg);
            break;
        case MRLBM_STORAGE_BF16:
            inlet_density_kernel<__nv_bfloat16><<<1, kInletThreads, 0, s>>>(ga, buf, state, slot, n_avg);
            break;
        case MRLBM_STORAGE_F16_U32:
            inlet_density_kernel<HybridWord><<<1, kInletThreads, 0, s>>>(ga, buf, state, slot, n_avg);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_surface_pressure(const StepArgs *ga, int buf, int storage, int wall, int nb, double *avg, int n_avg,
                                    cudaStream_t s) {
    if (nb <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((nb + 127) / 128);
    switch (storage) {
        case MRLBM_STORAGE_F32: surface_pressure_kernel<float><<<blocks, 128, 0, s>>>(ga, buf, wall, avg, n_avg); break;
        case MRLBM_STORAGE_F16: surface_pressure_kernel<__half><<<blocks, 128, 0, s>>>(ga, buf, wall, avg, n_avg); break;
        case MRLBM_STORAGE_BF16:
            surface_pressure_kernel<__nv_bfloat16><<<blocks, 128, 0, s>>>(ga, buf, wall, avg, n_avg);
            break;
        case MRLBM_STORAGE_F16_U32:
            surface_pressure_kernel<HybridWord><<<blocks, 128, 0, s>>>(ga, buf, wall, avg, n_avg);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace mrlbm
