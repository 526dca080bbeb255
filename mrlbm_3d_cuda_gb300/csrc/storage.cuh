// Moment storage in HBM: 10 field-major planes (rho - rho0, ux, uy, uz, mxx, myy, mzz, mxy,
// mxz, myz), each `fs` elements, lexicographic node order.  FP32, or FP16 / BF16 holding
// scaled deviations from the rest state (rho0, u = 0, m = 0).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <type_traits>

#include "kernels.h"
#include "lbm_device.cuh"

namespace mrlbm {

template <typename S>
__device__ __forceinline__ float to_f(S v);
template <>
__device__ __forceinline__ float to_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ float to_f<__half>(__half v) { return __half2float(v); }
template <>
__device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

template <typename S>
__device__ __forceinline__ S from_f(float v);
template <>
__device__ __forceinline__ float from_f<float>(float v) { return v; }
template <>
__device__ __forceinline__ __half from_f<__half>(float v) { return __float2half_rn(v); }
template <>
__device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }

__host__ __device__ constexpr int scale_class(int field) { return field == 0 ? 0 : (field < 4 ? 1 : 2); }

// Raw stored values -> moments (full rho).
template <typename S>
__device__ __forceinline__ Mom decode(const float v[10], float rho0, const StorageScale &sc) {
    Mom m;
    if constexpr (std::is_same<S, float>::value) {
        m.rho = rho0 + v[0];
        m.ux = v[1]; m.uy = v[2]; m.uz = v[3];
        m.mxx = v[4]; m.myy = v[5]; m.mzz = v[6];
        m.mxy = v[7]; m.mxz = v[8]; m.myz = v[9];
    } else {
        m.rho = rho0 + v[0] * sc.is[0];
        m.ux = v[1] * sc.is[1]; m.uy = v[2] * sc.is[1]; m.uz = v[3] * sc.is[1];
        m.mxx = v[4] * sc.is[2]; m.myy = v[5] * sc.is[2]; m.mzz = v[6] * sc.is[2];
        m.mxy = v[7] * sc.is[2]; m.mxz = v[8] * sc.is[2]; m.myz = v[9] * sc.is[2];
    }
    return m;
}

template <typename S>
__device__ __forceinline__ void load_raw(const S *__restrict__ base, int64_t fs, int64_t node, float v[10]) {
#pragma unroll
    for (int k = 0; k < 10; ++k) v[k] = to_f<S>(base[k * fs + node]);
}

template <typename S>
__device__ __forceinline__ Mom load_mom(const S *__restrict__ base, int64_t fs, int64_t node, float rho0,
                                        const StorageScale &sc) {
    float v[10];
    load_raw<S>(base, fs, node, v);
    return decode<S>(v, rho0, sc);
}

template <typename S>
__device__ __forceinline__ void store_mom(S *__restrict__ base, int64_t fs, int64_t node, const Mom &m, float rho0,
                                          const StorageScale &sc) {
    if constexpr (std::is_same<S, float>::value) {
        base[0 * fs + node] = m.rho - rho0;
        base[1 * fs + node] = m.ux;
        base[2 * fs + node] = m.uy;
        base[3 * fs + node] = m.uz;
        base[4 * fs + node] = m.mxx;
        base[5 * fs + node] = m.myy;
        base[6 * fs + node] = m.mzz;
        base[7 * fs + node] = m.mxy;
        base[8 * fs + node] = m.mxz;
        base[9 * fs + node] = m.myz;
    } else {
        base[0 * fs + node] = from_f<S>((m.rho - rho0) * sc.s[0]);
        base[1 * fs + node] = from_f<S>(m.ux * sc.s[1]);
        base[2 * fs + node] = from_f<S>(m.uy * sc.s[1]);
        base[3 * fs + node] = from_f<S>(m.uz * sc.s[1]);
        base[4 * fs + node] = from_f<S>(m.mxx * sc.s[2]);
        base[5 * fs + node] = from_f<S>(m.myy * sc.s[2]);
        base[6 * fs + node] = from_f<S>(m.mzz * sc.s[2]);
        base[7 * fs + node] = from_f<S>(m.mxy * sc.s[2]);
        base[8 * fs + node] = from_f<S>(m.mxz * sc.s[2]);
        base[9 * fs + node] = from_f<S>(m.myz * sc.s[2]);
    }
}

}  // namespace mrlbm
