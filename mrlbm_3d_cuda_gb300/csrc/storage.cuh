// Moment storage in HBM, x-blocked and field-interleaved: the 32 nodes x = 32 b .. 32 b + 31 of
// one (y, z) row keep their 10 fields (rho - rho0, ux, uy, uz, mxx, myy, mzz, mxy, mxz, myz)
// in one contiguous run of 10 x 32 values, and all 10 fields of a node sit at constant
// offsets from one address.  FP32 keeps one field per 128-byte line (a warp moves a field of
// its row per access); FP16 / BF16 hold scaled deviations from the rest state (rho0, u = 0,
// m = 0) with the field pairs (2j, 2j+1) of a node in one 32-bit word, so a warp moves two
// fields of its row per 128-byte access (kernels.h: aos_index, field_offset).
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

// Storage that keeps scaled deviations (every mode but FP32): the emit computes u and m with
// their storage scales folded in and stores through store_scaled*.
template <typename S>
constexpr bool kScaled = !std::is_same<S, float>::value;
template <typename S>
constexpr bool kHybrid = std::is_same<S, HybridWord>::value;

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
        m.rho = __fmaf_rn(v[0], sc.is[0], rho0);  // one rounding in every caller
        m.ux = v[1] * sc.is[1]; m.uy = v[2] * sc.is[1]; m.uz = v[3] * sc.is[1];
        m.mxx = v[4] * sc.is[2]; m.myy = v[5] * sc.is[2]; m.mzz = v[6] * sc.is[2];
        m.mxy = v[7] * sc.is[2]; m.mxz = v[8] * sc.is[2]; m.myz = v[9] * sc.is[2];
    }
    return m;
}

// Stored words of one node as loaded, decoded only where they are used: ten floats for FP32,
// five 32-bit words (the field pairs) for 16-bit storage.  Prefetching these instead of decoded
// floats keeps the 16-bit prefetch in flight (a conversion right after the load would wait
// for it) and in half the registers.
template <typename S>
struct Raw {
    float v[10];
};
template <>
struct Raw<__half> {
    uint32_t w[5];
};
template <>
struct Raw<__nv_bfloat16> {
    uint32_t w[5];
};
template <>
struct Raw<HybridWord> {
    float u[3];     // ux, uy, uz (FP32, unscaled)
    uint32_t w[4];  // FP16 pairs (rho', mxx), (myy, mzz), (mxy, mxz), (myz, -)
};

// Populations of a node from its raw stored values: FP32 through the moments; 16-bit storage
// with the storage scales folded into the Hermite factors, so u and m are never unscaled.
template <typename S>
__device__ __forceinline__ void rebuild(const float v[10], float rho0, const StorageScale &sc, float f[27]) {
    if constexpr (std::is_same<S, float>::value) {
        reconstruct(decode<S>(v, rho0, sc), f);
    } else {
        Mom m;
        m.rho = __fmaf_rn(v[0], sc.is[0], rho0);
        m.ux = v[1]; m.uy = v[2]; m.uz = v[3];
        m.mxx = v[4]; m.myy = v[5]; m.mzz = v[6];
        m.mxy = v[7]; m.mxz = v[8]; m.myz = v[9];
        reconstruct_h(m, __fmul_rn(3.0f, sc.is[1]), __fmul_rn(1.5f, sc.is[2]), __fmul_rn(4.5f, sc.is[2]),
                      __fmul_rn(9.0f, sc.is[2]), f);
    }
}

// Two 16-bit values of one 32-bit word (lower address first) <-> two floats.
template <typename S>
__device__ __forceinline__ float2 pair_to_f(uint32_t w);
template <>
__device__ __forceinline__ float2 pair_to_f<__half>(uint32_t w) {
    __half2 h;
    memcpy(&h, &w, 4);
    return __half22float2(h);
}
template <>
__device__ __forceinline__ float2 pair_to_f<__nv_bfloat16>(uint32_t w) {
    __nv_bfloat162 h;
    memcpy(&h, &w, 4);
    return __bfloat1622float2(h);
}
template <typename S>
__device__ __forceinline__ uint32_t pair_from_f(float a, float b);
template <>
__device__ __forceinline__ uint32_t pair_from_f<__half>(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    uint32_t w;
    memcpy(&w, &h, 4);
    return w;
}
template <>
__device__ __forceinline__ uint32_t pair_from_f<__nv_bfloat16>(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    uint32_t w;
    memcpy(&w, &h, 4);
    return w;
}

// Stochastic rounding of two floats to one packed 16-bit pair with Blackwell's cvt.rs:
// `lo` goes to the lower half (lower address), `hi` to the upper half; `rbits` are the
// random bits that decide each rounding direction.
template <typename S>
__device__ __forceinline__ uint32_t pair_from_f_sr(float lo, float hi, uint32_t rbits);
template <>
__device__ __forceinline__ uint32_t pair_from_f_sr<__half>(float lo, float hi, uint32_t rbits) {
    uint32_t d;
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
    return d;
}
template <>
__device__ __forceinline__ uint32_t pair_from_f_sr<__nv_bfloat16>(float lo, float hi, uint32_t rbits) {
    uint32_t d;
    asm("cvt.rs.bf16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
    return d;
}

// 32-bit integer hash ("lowbias32" from C. Wellons' hash prospector): avalanching, so the
// node index, field pair and step number give independent-looking random bits.
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
// Random-bit key of node (x, y, z) at the step with seed mix32(step): one per node and step.
__device__ __forceinline__ uint32_t sr_key(uint32_t step_seed, int x, int y, int z, int nx, int ny) {
    return mix32((((uint32_t)z * (uint32_t)ny + (uint32_t)y) * (uint32_t)nx + (uint32_t)x) ^ step_seed);
}
__device__ __forceinline__ uint32_t sr_step_seed(uint32_t step) { return mix32(step * 0x9e3779b9u + 0x632be5abu); }

// `ai` is the element index of field 0 of a node (aos_index); field k sits at
// ai + field_offset(k): 32 k for FP32, 64 (k / 2) + k % 2 for FP16 / BF16 (ai is even there).
// Hybrid: the 10 stored values of a node from its 3 FP32 words and 4 FP16 pair words.
__device__ __forceinline__ void hybrid_values(const float u[3], const uint32_t w[4], float v[10]) {
    const float2 a = pair_to_f<__half>(w[0]), b = pair_to_f<__half>(w[1]), c = pair_to_f<__half>(w[2]),
                 d = pair_to_f<__half>(w[3]);
    v[0] = a.x;
    v[1] = u[0]; v[2] = u[1]; v[3] = u[2];
    v[4] = a.y; v[5] = b.x; v[6] = b.y; v[7] = c.x; v[8] = c.y; v[9] = d.x;
}

template <typename S>
__device__ __forceinline__ void load_raw(const S *__restrict__ base, int64_t ai, float v[10]) {
    if constexpr (std::is_same<S, float>::value) {
        const float *p = base + ai;
#pragma unroll
        for (int k = 0; k < 10; ++k) v[k] = p[k * kXBlock];
    } else if constexpr (kHybrid<S>) {
        const uint32_t *p = reinterpret_cast<const uint32_t *>(base + ai);
        float u[3];
        uint32_t w[4];
#pragma unroll
        for (int k = 0; k < 3; ++k) u[k] = __uint_as_float(p[k * kXBlock]);
#pragma unroll
        for (int k = 0; k < 4; ++k) w[k] = p[(3 + k) * kXBlock];
        hybrid_values(u, w, v);
    } else {
        const uint32_t *p = reinterpret_cast<const uint32_t *>(base + ai);
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            const float2 f = pair_to_f<S>(p[j * kXBlock]);
            v[2 * j] = f.x;
            v[2 * j + 1] = f.y;
        }
    }
}

// Load the stored words of a node without decoding them.
template <typename S>
__device__ __forceinline__ void load_words(const S *__restrict__ base, int64_t ai, Raw<S> &r) {
    if constexpr (std::is_same<S, float>::value) {
        const float *p = base + ai;
#pragma unroll
        for (int k = 0; k < 10; ++k) r.v[k] = p[k * kXBlock];
    } else if constexpr (kHybrid<S>) {
        const uint32_t *p = reinterpret_cast<const uint32_t *>(base + ai);
#pragma unroll
        for (int k = 0; k < 3; ++k) r.u[k] = __uint_as_float(p[k * kXBlock]);
#pragma unroll
        for (int k = 0; k < 4; ++k) r.w[k] = p[(3 + k) * kXBlock];
    } else {
        const uint32_t *p = reinterpret_cast<const uint32_t *>(base + ai);
#pragma unroll
        for (int j = 0; j < 5; ++j) r.w[j] = p[j * kXBlock];
    }
}

// Populations of a node from its loaded words (rebuild of the decoded values).
template <typename S>
__device__ __forceinline__ void rebuild(const Raw<S> &r, float rho0, const StorageScale &sc, float f[27]) {
    if constexpr (std::is_same<S, float>::value) {
        rebuild<S>(r.v, rho0, sc, f);
    } else if constexpr (kHybrid<S>) {
        float v[10];
        hybrid_values(r.u, r.w, v);
        rebuild<S>(v, rho0, sc, f);
    } else {
        float v[10];
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            const float2 t = pair_to_f<S>(r.w[j]);
            v[2 * j] = t.x;
            v[2 * j + 1] = t.y;
        }
        rebuild<S>(v, rho0, sc, f);
    }
}

// Moments (full rho) of a node from its loaded words: load_mom without the load.
template <typename S>
__device__ __forceinline__ Mom decode_words(const Raw<S> &r, float rho0, const StorageScale &sc) {
    float v[10];
    if constexpr (std::is_same<S, float>::value) {
#pragma unroll
        for (int k = 0; k < 10; ++k) v[k] = r.v[k];
    } else if constexpr (kHybrid<S>) {
        hybrid_values(r.u, r.w, v);
    } else {
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            const float2 t = pair_to_f<S>(r.w[j]);
            v[2 * j] = t.x;
            v[2 * j + 1] = t.y;
        }
    }
    return decode<S>(v, rho0, sc);
}

template <typename S>
__device__ __forceinline__ Mom load_mom(const S *__restrict__ base, int64_t ai, float rho0, const StorageScale &sc) {
    float v[10];
    load_raw<S>(base, ai, v);
    return decode<S>(v, rho0, sc);
}

template <typename S>
__device__ __forceinline__ void store_mom(S *__restrict__ base, int64_t ai, const Mom &m, float rho0,
                                          const StorageScale &sc) {
    S *p = base + ai;
    if constexpr (std::is_same<S, float>::value) {
        p[0 * kXBlock] = m.rho - rho0;
        p[1 * kXBlock] = m.ux;
        p[2 * kXBlock] = m.uy;
        p[3 * kXBlock] = m.uz;
        p[4 * kXBlock] = m.mxx;
        p[5 * kXBlock] = m.myy;
        p[6 * kXBlock] = m.mzz;
        p[7 * kXBlock] = m.mxy;
        p[8 * kXBlock] = m.mxz;
        p[9 * kXBlock] = m.myz;
    } else if constexpr (kHybrid<S>) {
        uint32_t *w = reinterpret_cast<uint32_t *>(p);
        w[0 * kXBlock] = __float_as_uint(m.ux * sc.s[1]);
        w[1 * kXBlock] = __float_as_uint(m.uy * sc.s[1]);
        w[2 * kXBlock] = __float_as_uint(m.uz * sc.s[1]);
        w[3 * kXBlock] = pair_from_f<__half>((m.rho - rho0) * sc.s[0], m.mxx * sc.s[2]);
        w[4 * kXBlock] = pair_from_f<__half>(m.myy * sc.s[2], m.mzz * sc.s[2]);
        w[5 * kXBlock] = pair_from_f<__half>(m.mxy * sc.s[2], m.mxz * sc.s[2]);
        w[6 * kXBlock] = pair_from_f<__half>(m.myz * sc.s[2], 0.0f);
    } else {
        uint32_t *w = reinterpret_cast<uint32_t *>(p);
        w[0 * kXBlock] = pair_from_f<S>((m.rho - rho0) * sc.s[0], m.ux * sc.s[1]);
        w[1 * kXBlock] = pair_from_f<S>(m.uy * sc.s[1], m.uz * sc.s[1]);
        w[2 * kXBlock] = pair_from_f<S>(m.mxx * sc.s[2], m.myy * sc.s[2]);
        w[3 * kXBlock] = pair_from_f<S>(m.mzz * sc.s[2], m.mxy * sc.s[2]);
        w[4 * kXBlock] = pair_from_f<S>(m.mxz * sc.s[2], m.myz * sc.s[2]);
    }
}

// store_mom with stochastic rounding of the 16-bit pairs (random bits from `key`, one hash per
// pair); FP32 storage has nothing to round
template <typename S>
__device__ __forceinline__ void store_mom_sr(S *__restrict__ base, int64_t ai, const Mom &m, float rho0,
                                             const StorageScale &sc, uint32_t key) {
    if constexpr (std::is_same<S, float>::value) {
        store_mom<S>(base, ai, m, rho0, sc);
    } else if constexpr (kHybrid<S>) {
        uint32_t *w = reinterpret_cast<uint32_t *>(base + ai);
        w[0 * kXBlock] = __float_as_uint(m.ux * sc.s[1]);
        w[1 * kXBlock] = __float_as_uint(m.uy * sc.s[1]);
        w[2 * kXBlock] = __float_as_uint(m.uz * sc.s[1]);
        w[3 * kXBlock] = pair_from_f_sr<__half>((m.rho - rho0) * sc.s[0], m.mxx * sc.s[2], mix32(key));
        w[4 * kXBlock] = pair_from_f_sr<__half>(m.myy * sc.s[2], m.mzz * sc.s[2], mix32(key + 0x9e3779b9u));
        w[5 * kXBlock] = pair_from_f_sr<__half>(m.mxy * sc.s[2], m.mxz * sc.s[2], mix32(key + 0x3c6ef372u));
        w[6 * kXBlock] = pair_from_f_sr<__half>(m.myz * sc.s[2], 0.0f, mix32(key + 0xdaa66d2bu));
    } else {
        uint32_t *w = reinterpret_cast<uint32_t *>(base + ai);
        w[0 * kXBlock] = pair_from_f_sr<S>((m.rho - rho0) * sc.s[0], m.ux * sc.s[1], mix32(key));
        w[1 * kXBlock] = pair_from_f_sr<S>(m.uy * sc.s[1], m.uz * sc.s[1], mix32(key + 0x9e3779b9u));
        w[2 * kXBlock] = pair_from_f_sr<S>(m.mxx * sc.s[2], m.myy * sc.s[2], mix32(key + 0x3c6ef372u));
        w[3 * kXBlock] = pair_from_f_sr<S>(m.mzz * sc.s[2], m.mxy * sc.s[2], mix32(key + 0xdaa66d2bu));
        w[4 * kXBlock] = pair_from_f_sr<S>(m.mxz * sc.s[2], m.myz * sc.s[2], mix32(key + 0x78dde6e4u));
    }
}

// Stores of moments already held with the storage scales (u s_u, m s_m; rho as the full
// density), as the bulk emit of the step kernel computes them for 16-bit storage.
template <typename S>
__device__ __forceinline__ void store_scaled(S *__restrict__ base, int64_t ai, const Mom &m, float rho0,
                                             const StorageScale &sc) {
    static_assert(!std::is_same<S, float>::value, "FP32 storage holds physical moments");
    uint32_t *w = reinterpret_cast<uint32_t *>(base + ai);
    if constexpr (kHybrid<S>) {
        w[0 * kXBlock] = __float_as_uint(m.ux);
        w[1 * kXBlock] = __float_as_uint(m.uy);
        w[2 * kXBlock] = __float_as_uint(m.uz);
        w[3 * kXBlock] = pair_from_f<__half>((m.rho - rho0) * sc.s[0], m.mxx);
        w[4 * kXBlock] = pair_from_f<__half>(m.myy, m.mzz);
        w[5 * kXBlock] = pair_from_f<__half>(m.mxy, m.mxz);
        w[6 * kXBlock] = pair_from_f<__half>(m.myz, 0.0f);
        return;
    }
    w[0 * kXBlock] = pair_from_f<S>((m.rho - rho0) * sc.s[0], m.ux);
    w[1 * kXBlock] = pair_from_f<S>(m.uy, m.uz);
    w[2 * kXBlock] = pair_from_f<S>(m.mxx, m.myy);
    w[3 * kXBlock] = pair_from_f<S>(m.mzz, m.mxy);
    w[4 * kXBlock] = pair_from_f<S>(m.mxz, m.myz);
}
template <typename S>
__device__ __forceinline__ void store_scaled_sr(S *__restrict__ base, int64_t ai, const Mom &m, float rho0,
                                                const StorageScale &sc, uint32_t key) {
    static_assert(!std::is_same<S, float>::value, "FP32 storage holds physical moments");
    uint32_t *w = reinterpret_cast<uint32_t *>(base + ai);
    if constexpr (kHybrid<S>) {
        w[0 * kXBlock] = __float_as_uint(m.ux);
        w[1 * kXBlock] = __float_as_uint(m.uy);
        w[2 * kXBlock] = __float_as_uint(m.uz);
        w[3 * kXBlock] = pair_from_f_sr<__half>((m.rho - rho0) * sc.s[0], m.mxx, mix32(key));
        w[4 * kXBlock] = pair_from_f_sr<__half>(m.myy, m.mzz, mix32(key + 0x9e3779b9u));
        w[5 * kXBlock] = pair_from_f_sr<__half>(m.mxy, m.mxz, mix32(key + 0x3c6ef372u));
        w[6 * kXBlock] = pair_from_f_sr<__half>(m.myz, 0.0f, mix32(key + 0xdaa66d2bu));
        return;
    }
    w[0 * kXBlock] = pair_from_f_sr<S>((m.rho - rho0) * sc.s[0], m.ux, mix32(key));
    w[1 * kXBlock] = pair_from_f_sr<S>(m.uy, m.uz, mix32(key + 0x9e3779b9u));
    w[2 * kXBlock] = pair_from_f_sr<S>(m.mxx, m.myy, mix32(key + 0x3c6ef372u));
    w[3 * kXBlock] = pair_from_f_sr<S>(m.mzz, m.mxy, mix32(key + 0xdaa66d2bu));
    w[4 * kXBlock] = pair_from_f_sr<S>(m.mxz, m.myz, mix32(key + 0x78dde6e4u));
}

// One stored field of a node (the stored, scaled value) and its store: the layout of each
// mode (field_offset for FP32 / FP16 / BF16; the hybrid mode's FP32 words and FP16 halves).
template <typename S>
__device__ __forceinline__ float load_field(const S *__restrict__ base, int64_t ai, int f) {
    if constexpr (kHybrid<S>) {
        const uint32_t *p = reinterpret_cast<const uint32_t *>(base + ai);
        if (f >= 1 && f <= 3) return __uint_as_float(p[(f - 1) * kXBlock]);
        const int k = f == 0 ? 0 : f - 3;  // half index among rho', mxx, myy, ..., myz
        const __half *h = reinterpret_cast<const __half *>(p + (3 + (k >> 1)) * kXBlock);
        return __half2float(h[k & 1]);
    } else {
        return to_f<S>(base[ai + field_offset(f, (int)sizeof(S))]);
    }
}
template <typename S>
__device__ __forceinline__ void store_field(S *__restrict__ base, int64_t ai, int f, float v) {
    if constexpr (kHybrid<S>) {
        uint32_t *p = reinterpret_cast<uint32_t *>(base + ai);
        if (f >= 1 && f <= 3) {
            p[(f - 1) * kXBlock] = __float_as_uint(v);
            return;
        }
        const int k = f == 0 ? 0 : f - 3;
        __half *h = reinterpret_cast<__half *>(p + (3 + (k >> 1)) * kXBlock);
        h[k & 1] = __float2half_rn(v);
    } else {
        base[ai + field_offset(f, (int)sizeof(S))] = from_f<S>(v);
    }
}

}  // namespace mrlbm
