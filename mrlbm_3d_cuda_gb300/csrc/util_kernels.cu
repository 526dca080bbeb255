// Initial conditions and host-facing layout conversion.
//
// Reference (paths inside sakthi-lbm/MRLBM_3D_CUDA):
//   gpu_initialize_Moments_GhostInterface  MRLBM_3D/src/solver/initializeLBM.cu:39-121
//   get_noise                              MRLBM_3D/src/solver/initializeLBM.cu:24-37
// The reference initialiser builds "equilibrium" populations from __constant__ tables that
// are uploaded only later (simulation.cu:22 runs before :30), so the populations and hence
// m_ij come out zero; MRLBM_INIT_REFERENCE_NOISE reproduces that state bit for bit,
// including the hash noise keyed on the reference's tiled node index.
#include <cmath>

#include "mrlbm_internal.h"
#include "storage.cuh"

namespace mrlbm {
namespace {

// 32-bit integer hash (Thomas Wang's avalanche sequence) mapped to [-scale, scale], as the
// reference's get_noise.
__device__ __forceinline__ float hash_noise(unsigned int seed, float scale) {
    seed = (seed ^ 61u) ^ (seed >> 16);
    seed *= 9u;
    seed = seed ^ (seed >> 4);
    seed *= 0x27d4eb2du;
    seed = seed ^ (seed >> 15);
    const float r = (float)(seed & 0x7FFFFFFFu) / (float)0x7FFFFFFF;
    return scale * (2.0f * r - 1.0f);
}

template <typename S>
__global__ void init_kernel(const InitArgs a) {
    const int64_t n = (int64_t)a.nx * a.ny * a.nz;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % a.nx), y = (int)((i / a.nx) % a.ny), z = (int)(i / ((int64_t)a.nx * a.ny));
    Mom m;
    m.rho = a.rho0;
    m.ux = m.uy = m.uz = 0.f;
    m.mxx = m.myy = m.mzz = m.mxy = m.mxz = m.myz = 0.f;
    switch (a.kind) {
        case MRLBM_INIT_REFERENCE_NOISE: {
            const float pi_f = 3.14159265358979323846f;
            const float noise_scale = 1e-4f * a.u_max;
            const int64_t ridx = ref_tiled_index(x, y, z, a.nx, a.ny);
            const double s = sin(2.0 * (double)pi_f * (double)(float)z / (double)(float)a.nz);
            m.uz = (float)(1e-4 * (double)a.u_max * s + (double)hash_noise((unsigned int)(ridx + 67890), noise_scale));
            break;
        }
        case MRLBM_INIT_REST: break;
        case MRLBM_INIT_TAYLOR_GREEN: {
            const double u0 = a.p[0], L = a.p[1];
            const double X = x / L, Y = y / L, Z = z / L;
            const double u = u0 * sin(X) * cos(Y) * cos(Z);
            const double v = -u0 * cos(X) * sin(Y) * cos(Z);
            const double p = (double)a.rho0 * u0 * u0 / 16.0 * (cos(2.0 * X) + cos(2.0 * Y)) * (cos(2.0 * Z) + 2.0);
            m.rho = (float)((double)a.rho0 + 3.0 * p);
            m.ux = (float)u;
            m.uy = (float)v;
            m.uz = 0.f;
            m.mxx = (float)(u * u);
            m.myy = (float)(v * v);
            m.mxy = (float)(u * v);
            break;
        }
        case MRLBM_INIT_UNIFORM:
        case MRLBM_INIT_NOISY_UNIFORM: {
            double u = a.p[0], v = a.p[1], w = a.p[2];
            if (a.kind == MRLBM_INIT_NOISY_UNIFORM) {
                const double amp = a.p[3];
                const unsigned int seed = (unsigned int)a.p[4];
                const double umag = sqrt(u * u + v * v + w * w);
                const unsigned int base = (unsigned int)i * 3u + seed;
                u += umag * amp * hash_noise(base + 0u, 1.0f);
                v += umag * amp * hash_noise(base + 1u, 1.0f);
                w += umag * amp * hash_noise(base + 2u, 1.0f);
            }
            m.ux = (float)u; m.uy = (float)v; m.uz = (float)w;
            m.mxx = (float)(u * u); m.myy = (float)(v * v); m.mzz = (float)(w * w);
            m.mxy = (float)(u * v); m.mxz = (float)(u * w); m.myz = (float)(v * w);
            break;
        }
        default: break;
    }
    const int64_t ai = aos_at<S>(x, y, z, (a.nx + kXBlock - 1) / kXBlock, a.ny);
    store_mom<S>((S *)a.m_a, ai, m, a.rho0, a.sc);
    store_mom<S>((S *)a.m_b, ai, m, a.rho0, a.sc);
}

template <typename S>
__global__ void convert_kernel(const S *src, S *dst_a, S *dst_b, float *f32, uint32_t mask, int layout,
                               int nx, int ny, int nz, StorageScale sc, int dir) {
    const int64_t n = (int64_t)nx * ny * nz;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((int64_t)nx * ny));
    const int64_t h = layout == MRLBM_LAYOUT_REF_TILED ? ref_tiled_index(x, y, z, nx, ny) : i;
    const int64_t ai = aos_at<S>(x, y, z, (nx + kXBlock - 1) / kXBlock, ny);
    int slot = 0;
    for (int f = 0; f < 10; ++f) {
        if (!(mask & (1u << f))) continue;
        const float s = sc.s[scale_class(f)], is = sc.is[scale_class(f)];
        const bool lowp = kScaled<S>;
        if (dir == 0) {
            const float v = load_field<S>(src, ai, f);
            f32[(int64_t)slot * n + h] = lowp ? v * is : v;
        } else {
            const float v = f32[(int64_t)slot * n + h];
            store_field<S>(dst_a, ai, f, lowp ? v * s : v);
            if (dst_b) store_field<S>(dst_b, ai, f, lowp ? v * s : v);
        }
        ++slot;
    }
}

// One step further along the stochastic-rounding random sequence: the step counter of one
// case, or of every case of a batch that rounds stochastically.
__global__ void sr_tick_kernel(uint32_t *ctr) { ++*ctr; }
__global__ void sr_tick_cases_kernel(const StepArgs *const *cases, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && cases[i]->sr_step) ++*const_cast<uint32_t *>(cases[i]->sr_step);
}

}  // namespace

cudaError_t launch_sr_tick(uint32_t *ctr, cudaStream_t s) {
    sr_tick_kernel<<<1, 1, 0, s>>>(ctr);
    return cudaGetLastError();
}

cudaError_t launch_sr_tick_cases(const StepArgs *const *cases, int n, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    sr_tick_cases_kernel<<<(n + 127) / 128, 128, 0, s>>>(cases, n);
    return cudaGetLastError();
}

cudaError_t launch_init(const InitArgs &a, int storage, cudaStream_t s) {
    const int64_t n = (int64_t)a.nx * a.ny * a.nz;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    switch (storage) {
        case MRLBM_STORAGE_F32: init_kernel<float><<<blocks, 256, 0, s>>>(a); break;
        case MRLBM_STORAGE_F16: init_kernel<__half><<<blocks, 256, 0, s>>>(a); break;
        case MRLBM_STORAGE_BF16: init_kernel<__nv_bfloat16><<<blocks, 256, 0, s>>>(a); break;
        case MRLBM_STORAGE_F16_U32: init_kernel<HybridWord><<<blocks, 256, 0, s>>>(a); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_convert(const void *src, void *dst_a, void *dst_b, float *f32, uint32_t field_mask,
                           int layout, int nx, int ny, int nz, int storage, const StorageScale &sc, int dir,
                           cudaStream_t s) {
    const int64_t n = (int64_t)nx * ny * nz;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    switch (storage) {
        case MRLBM_STORAGE_F32:
            convert_kernel<float><<<blocks, 256, 0, s>>>((const float *)src, (float *)dst_a, (float *)dst_b, f32,
                                                         field_mask, layout, nx, ny, nz, sc, dir);
            break;
        case MRLBM_STORAGE_F16:
            convert_kernel<__half><<<blocks, 256, 0, s>>>((const __half *)src, (__half *)dst_a, (__half *)dst_b, f32,
                                                          field_mask, layout, nx, ny, nz, sc, dir);
            break;
        case MRLBM_STORAGE_BF16:
            convert_kernel<__nv_bfloat16><<<blocks, 256, 0, s>>>((const __nv_bfloat16 *)src, (__nv_bfloat16 *)dst_a,
                                                                 (__nv_bfloat16 *)dst_b, f32, field_mask, layout,
                                                                 nx, ny, nz, sc, dir);
            break;
        case MRLBM_STORAGE_F16_U32:
            convert_kernel<HybridWord><<<blocks, 256, 0, s>>>((const HybridWord *)src, (HybridWord *)dst_a,
                                                                 (HybridWord *)dst_b, f32, field_mask, layout,
                                                                 nx, ny, nz, sc, dir);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace mrlbm
