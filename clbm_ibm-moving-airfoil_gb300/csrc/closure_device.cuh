// closure_device.cuh -- device functions of the learned sub-grid closure: the moment
// features of a cell, the closure relaxation of its third- and fourth-order central
// moments, and the pieces of the 19 -> 32 -> 32 -> 1 network shared by the fused
// stream-collide kernel, the training kernel and the self tests.
#pragma once

#include <cuda_bf16.h>

#include "lbm_device.cuh"
#include "tc.cuh"

namespace clbm {
namespace closure {

// Moments of one cell about its velocity u = m / rho (closure cells carry no body force).
struct CMom {
    float r;        // density
    float u, v, w;  // velocity
    float x[kIn];   // non-equilibrium central moments / rho, in the M_raw order
                    // (config_moving.py:62-68): 000, 100, 010, 001, 110, 101, 011,
                    // 200, 020, 002, 210, 120, 201, 021, 102, 012, 220, 202, 022
};

// Raw moments of a population vector up to the fourth order present in D3Q19, over a
// value type T (F1: one cell; V2: two cells in packed f32x2 arithmetic). DEV: f holds
// deviations f - w; the weights' part of the even moments is kept apart (sum w = 1,
// sum w e_a^2 = 1/3, sum w e_a^2 e_b^2 = 1/9; odd moments of w vanish).
template <class T>
struct RawT {
    T R0;                      // sum f (deviations: sum of deviations)
    T r;                       // density
    T mx, my, mz;
    T Pxx, Pyy, Pzz;           // second diagonal, without the weights' part
    T Mxx, Myy, Mzz;           // second diagonal, full
    T pxy, pxz, pyz;
    T M210, M120, M201, M021, M102, M012;
    T A220, A202, A022;        // fourth, without the weights' part
};

template <class T, bool DEV>
__device__ __forceinline__ RawT<T> raw_moments_t(const T (&f)[19]) {
    RawT<T> m;
    const T sx = f[1] + f[2], sy = f[3] + f[4], sz = f[5] + f[6];
    const T a = f[7] + f[8], b = f[9] + f[10], cc = f[11] + f[12], d = f[13] + f[14];
    const T e = f[15] + f[16], h = f[17] + f[18];
    m.R0 = f[0] + (sx + sy + sz) + (a + b) + (cc + d) + (e + h);
    m.mx = (f[1] - f[2]) + (f[7] - f[8]) + (f[9] - f[10]) + (f[11] - f[12]) + (f[13] - f[14]);
    m.my = (f[3] - f[4]) + (a - b) + (f[15] - f[16]) + (f[17] - f[18]);
    m.mz = (f[5] - f[6]) + (cc - d) + (e - h);
    m.Pxx = sx + (a + b) + (cc + d);
    m.Pyy = sy + (a + b) + (e + h);
    m.Pzz = sz + (cc + d) + (e + h);
    m.pxy = (f[7] + f[10]) - (f[8] + f[9]);
    m.pxz = (f[11] + f[14]) - (f[12] + f[13]);
    m.pyz = (f[15] + f[18]) - (f[16] + f[17]);
    // plane diagonals e = (+1,+1), (-1,+1), (+1,-1), (-1,-1) in each plane
    m.M210 = a - b;
    m.M120 = (f[7] - f[8]) + (f[9] - f[10]);
    m.M201 = cc - d;
    m.M102 = (f[11] - f[12]) + (f[13] - f[14]);
    m.M021 = e - h;
    m.M012 = (f[15] - f[16]) + (f[17] - f[18]);
    m.A220 = a + b;
    m.A202 = cc + d;
    m.A022 = e + h;
    const T s3 = vsplat(DEV ? 1.0f / 3.0f : 0.0f, f[0]);
    m.r = m.R0 + vsplat(DEV ? 1.0f : 0.0f, f[0]);
    m.Mxx = m.Pxx + s3;
    m.Myy = m.Pyy + s3;
    m.Mzz = m.Pzz + s3;
    return m;
}

// Non-equilibrium central moments about the velocity (u, v, w), times inv_rho (1 / rho_n),
// by the binomial expansion of sum f (e_x - u)^p (e_y - v)^q (e_z - w)^r; the equilibrium
// values subtracted are rho/3 (second diagonal) and rho/9 (fourth).
template <class T>
__device__ __forceinline__ void central_moments_t(const RawT<T>& m, T u, T v, T w, T inv_rho,
                                                  T (&x)[kIn]) {
    const T c2 = vsplat(2.0f, u), c4 = vsplat(4.0f, u);
    const T c13 = vsplat(1.0f / 3.0f, u), c19 = vsplat(1.0f / 9.0f, u);
    const T r = m.r, R0 = m.R0;
    const T mx = m.mx, my = m.my, mz = m.mz;
    const T ur = u * r, vr = v * r, wr = w * r;
    const T uu = u * u, vv = v * v, ww = w * w;
    const T uv2 = c2 * u * v, uw2 = c2 * u * w, vw2 = c2 * v * w;
    T k[kIn];
    k[0] = vsplat(0.0f, u);
    k[1] = mx - ur;
    k[2] = my - vr;
    k[3] = mz - wr;
    k[4] = m.pxy - u * my - v * mx + u * vr;
    k[5] = m.pxz - u * mz - w * mx + u * wr;
    k[6] = m.pyz - v * mz - w * my + v * wr;
    // k200 - r/3 = (P - R0/3) - 2u mx + u^2 r
    k[7] = (m.Pxx - R0 * c13) + u * (ur - c2 * mx);
    k[8] = (m.Pyy - R0 * c13) + v * (vr - c2 * my);
    k[9] = (m.Pzz - R0 * c13) + w * (wr - c2 * mz);
    // third order, e.g. k210 = M210 - 2u M110 - v M200 + 2uv M100 + u^2 M010 - u^2 v M000
    k[10] = m.M210 - c2 * u * m.pxy - v * m.Mxx + uv2 * mx + uu * (my - vr);
    k[11] = m.M120 - c2 * v * m.pxy - u * m.Myy + uv2 * my + vv * (mx - ur);
    k[12] = m.M201 - c2 * u * m.pxz - w * m.Mxx + uw2 * mx + uu * (mz - wr);
    k[13] = m.M021 - c2 * v * m.pyz - w * m.Myy + vw2 * my + vv * (mz - wr);
    k[14] = m.M102 - c2 * w * m.pxz - u * m.Mzz + uw2 * mz + ww * (mx - ur);
    k[15] = m.M012 - c2 * w * m.pyz - v * m.Mzz + vw2 * mz + ww * (my - vr);
    // fourth order, e.g. k220 - r/9 = (A220 - R0/9) - 2v M210 - 2u M120 + v^2 M200
    //   + u^2 M020 + 4uv M110 - 2uv^2 M100 - 2u^2 v M010 + u^2 v^2 M000
    k[16] = (m.A220 - R0 * c19) - c2 * v * m.M210 - c2 * u * m.M120 + vv * m.Mxx + uu * m.Myy +
            c4 * u * v * m.pxy - uv2 * v * mx - uv2 * u * my + uu * vv * r;
    k[17] = (m.A202 - R0 * c19) - c2 * w * m.M201 - c2 * u * m.M102 + ww * m.Mxx + uu * m.Mzz +
            c4 * u * w * m.pxz - uw2 * w * mx - uw2 * u * mz + uu * ww * r;
    k[18] = (m.A022 - R0 * c19) - c2 * w * m.M021 - c2 * v * m.M012 + ww * m.Myy + vv * m.Mzz +
            c4 * v * w * m.pyz - vw2 * w * my - vw2 * v * mz + vv * ww * r;
#pragma unroll
    for (int i = 0; i < kIn; ++i) x[i] = k[i] * inv_rho;
}

// Moments of a cell (or two) about its own velocity u = m / rho (closure cells carry no
// force): density r and the scaled non-equilibrium central moments x.
template <class T, bool DEV>
__device__ __forceinline__ void moments_full_t(const T (&f)[19], T& r, T (&x)[kIn]) {
    const RawT<T> m = raw_moments_t<T, DEV>(f);
    const T inv = vrcp(m.r);
    r = m.r;
    central_moments_t(m, m.mx * inv, m.my * inv, m.mz * inv, inv, x);
}

// Float forms of the above for one cell.
using Raw = RawT<F1>;

template <bool DEV>
__device__ __forceinline__ Raw raw_moments(const float (&f)[19]) {
    F1 t[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) t[q].x = f[q];
    return raw_moments_t<F1, DEV>(t);
}

__device__ __forceinline__ void central_moments(const Raw& m, float u, float v, float w, float rho_n,
                                                float (&x)[kIn]) {
    F1 t[kIn];
    central_moments_t(m, F1{u}, F1{v}, F1{w}, F1{1.0f / rho_n}, t);
#pragma unroll
    for (int i = 0; i < kIn; ++i) x[i] = t[i].x;
}

template <bool DEV>
__device__ __forceinline__ void moments_full(const float (&f)[19], CMom& c) {
    const Raw m = raw_moments<DEV>(f);
    const float inv = 1.0f / m.r.x;
    c.r = m.r.x;
    c.u = m.mx.x * inv;
    c.v = m.my.x * inv;
    c.w = m.mz.x * inv;
    central_moments(m, c.u, c.v, c.w, m.r.x, c.x);
}

// GELU, tanh form (Hendrycks and Gimpel), with the hardware tanh approximation.
__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float gelu(float z) {
    const float t = tanh_approx(0.7978845608028654f * (z + 0.044715f * z * z * z));
    return 0.5f * z * (1.0f + t);
}
// d gelu / dz for the same form.
__device__ __forceinline__ float gelu_grad(float z) {
    const float k = 0.7978845608028654f;
    const float t = tanh_approx(k * (z + 0.044715f * z * z * z));
    return 0.5f * (1.0f + t) + 0.5f * z * (1.0f - t * t) * k * (1.0f + 3.0f * 0.044715f * z * z);
}

__device__ __forceinline__ uint16_t bf16_bits(float x) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ float bf16_round(float x) {
    return __bfloat162float(__float2bfloat16_rn(x));
}

// Two values rounded to bf16 and packed (first in the low half), one conversion.
__device__ __forceinline__ uint32_t bf16x2_bits(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Write one row (32 values, rounded to bf16) of a K-major tile with 32 columns.
__device__ __forceinline__ void put_row32(unsigned char* tile, int row, const float (&v)[32]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        uint32_t wv[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) wv[t] = bf16x2_bits(v[8 * j + 2 * t], v[8 * j + 2 * t + 1]);
        *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(row, 8 * j, 32)) =
            make_uint4(wv[0], wv[1], wv[2], wv[3]);
    }
}

// GELU of two values with the packed f32x2 arithmetic and one half2 hardware tanh (the
// inference path; the training kernels use the float32 form above).
__device__ __forceinline__ V2 gelu2(V2 z) {
    const V2 zz = z * z;
    const V2 inner = z * vfma(vsplat(0.7978845608028654f * 0.044715f, z), zz, vsplat(0.7978845608028654f, z));
    const float2 in = vunpack(inner);
    const __half2 hin = __floats2half2_rn(in.x, in.y);
    uint32_t hout;
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(hout) : "r"(*reinterpret_cast<const uint32_t*>(&hin)));
    const float2 t = __half22float2(*reinterpret_cast<const __half2*>(&hout));
    const V2 hz = vsplat(0.5f, z) * z;
    return vfma(hz, vpack(t.x, t.y), hz);
}

// Network constants a block keeps in shared memory next to the BF16 weight images.
struct NetSmem {
    float mu[kIn], sinv[kIn];
    float b1[kHid], b2[kHid], w3[kHid];
    float b3, span, nu;
    int mode;
};

__device__ __forceinline__ void load_net(const float* __restrict__ p, NetSmem& n, int tid, int nthreads) {
    for (int i = tid; i < kIn; i += nthreads) {
        n.mu[i] = p[kMu + i];
        n.sinv[i] = p[kSinv + i];
    }
    for (int i = tid; i < kHid; i += nthreads) {
        n.b1[i] = p[kB1 + i];
        n.b2[i] = p[kB2 + i];
        n.w3[i] = bf16_round(p[kW3 + i]);
    }
    if (tid == 0) {
        n.b3 = p[kB3];
        n.span = p[kSpan];
        n.mode = (int)p[kMode];
        n.nu = p[kNu];
    }
}

// Moment orders (p, q, r) of the raw-moment set M_raw, in its row order
// (config_moving.py:62-68).
// (each order packed as 2 bits: p | q << 2 | r << 4)
__host__ __device__ constexpr int pqr_code(int i) {
    return i == 0 ? 0x00 : i == 1 ? 0x01 : i == 2 ? 0x04 : i == 3 ? 0x10 : i == 4 ? 0x05
         : i == 5 ? 0x11 : i == 6 ? 0x14 : i == 7 ? 0x02 : i == 8 ? 0x08 : i == 9 ? 0x20
         : i == 10 ? 0x06 : i == 11 ? 0x09 : i == 12 ? 0x12 : i == 13 ? 0x18 : i == 14 ? 0x21
         : i == 15 ? 0x24 : i == 16 ? 0x0A : i == 17 ? 0x22 : 0x28;
}

// Entry (moment i, population q) of M_raw: e_x^p e_y^q e_z^r, one of 0, +1, -1.
__device__ __forceinline__ int mraw_entry(int i, int q) {
    const int e[3] = {ex(q), ey(q), ez(q)};
    const int code = pqr_code(i);
    int v = 1;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        for (int k = 0; k < ((code >> (2 * a)) & 3); ++k) v *= e[a];
    return v;
}

// Raw moments of the stored deviations in the M_raw order (as the tensor cores return them:
// m_i = sum_q M_raw[i][q] h_q) turned into the cell's moments about its own velocity, the
// same arithmetic as moments_full<DEV = true> from there on.
__device__ __forceinline__ void moments_from_mraw(const float (&m)[32], CMom& c) {
    Raw r;
    r.R0.x = m[0];
    r.mx.x = m[1]; r.my.x = m[2]; r.mz.x = m[3];
    r.pxy.x = m[4]; r.pxz.x = m[5]; r.pyz.x = m[6];
    r.Pxx.x = m[7]; r.Pyy.x = m[8]; r.Pzz.x = m[9];
    r.M210.x = m[10]; r.M120.x = m[11]; r.M201.x = m[12];
    r.M021.x = m[13]; r.M102.x = m[14]; r.M012.x = m[15];
    r.A220.x = m[16]; r.A202.x = m[17]; r.A022.x = m[18];
    r.r.x = m[0] + 1.0f;
    r.Mxx.x = m[7] + 1.0f / 3.0f;
    r.Myy.x = m[8] + 1.0f / 3.0f;
    r.Mzz.x = m[9] + 1.0f / 3.0f;
    const float inv = 1.0f / r.r.x;
    c.r = r.r.x;
    c.u = r.mx.x * inv;
    c.v = r.my.x * inv;
    c.w = r.mz.x * inv;
    central_moments(r, c.u, c.v, c.w, r.r.x, c.x);
}

// Standardised features of a cell, padded to 32 with zeros.
__device__ __forceinline__ void standardise(const CMom& m, const NetSmem& n, float (&xs)[32]) {
#pragma unroll
    for (int i = 0; i < kIn; ++i) xs[i] = (m.x[i] - n.mu[i]) * n.sinv[i];
#pragma unroll
    for (int i = kIn; i < 32; ++i) xs[i] = 0.0f;
}

// Eddy-viscosity closure for the network output th = tanh(z3): effective viscosity
// nu 2^(span g), g = th for th >= 0 and th / 20 below (the network adds viscosity and may
// remove at most a factor 2^(-span/20)), its rate s = 1 / (1/2 + 3 nu_eff), and
// d nu_eff / d th.
constexpr float kEddyLeak = 0.05f;
__device__ __forceinline__ float eddy_nu(float nu, float span, float th, float* dnudth) {
    const float slope = th >= 0.0f ? 1.0f : kEddyLeak;
    const float nue = nu * exp2f(span * slope * th);
    if (dnudth) *dnudth = nue * 0.69314718f * span * slope;
    return nue;
}
__device__ __forceinline__ float eddy_rate(float nu, float span, float th) {
    return 1.0f / (0.5f + 3.0f * eddy_nu(nu, span, th, nullptr));
}

// Post-collision third-order central moments and fourth-order deviations from r/9 for
// the rate s_h: k3* = (1 - s_h) k3, k4* - r/9 = (1 - s_h)(k4 - r/9) (in the layout that
// collide_v<.., HO = true> takes). x holds the moments divided by r.
__device__ __forceinline__ void higher_order_post(const CMom& m, float sh, float (&ho)[9]) {
    const float g = (1.0f - sh) * m.r;
#pragma unroll
    for (int i = 0; i < 9; ++i) ho[i] = g * m.x[10 + i];
}

}  // namespace closure
}  // namespace clbm
