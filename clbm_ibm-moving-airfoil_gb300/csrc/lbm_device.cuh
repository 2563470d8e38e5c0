// lbm_device.cuh -- device functions of the stream-collide pass shared by the
// single-lattice kernels (lbm_kernels.cu) and the batched ensemble kernels (ensemble.cu).
#pragma once

#include <type_traits>

#include "clbm_internal.cuh"

namespace clbm {

// 3D Zou-He velocity inlet on the post-stream populations of an x = 0 cell,
// clbm_moving.py:266-294, in the same operation order with every operation explicitly
// rounded (no contraction), so the inlet column repeats the reference's float32 values.
__device__ __forceinline__ void zou_he(float (&v)[19], const Coef& c) {
    const float ux_in = c.ux_in, uy_in = c.uy_in;
    float S_known = v[0];
    S_known = __fadd_rn(S_known, v[3]);
    S_known = __fadd_rn(S_known, v[4]);
    S_known = __fadd_rn(S_known, v[5]);
    S_known = __fadd_rn(S_known, v[6]);
    S_known = __fadd_rn(S_known, v[15]);
    S_known = __fadd_rn(S_known, v[16]);
    S_known = __fadd_rn(S_known, v[17]);
    S_known = __fadd_rn(S_known, v[18]);
    float S_out = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(v[2], v[8]), v[10]), v[12]), v[14]);
    const float rho_in = __fdiv_rn(__fadd_rn(S_known, __fmul_rn(2.0f, S_out)), __fsub_rn(1.0f, ux_in));
    const float diff_y = __fsub_rn(v[3], v[4]);
    const float diff_z = __fsub_rn(v[5], v[6]);
    const float a23 = __fmul_rn(__fmul_rn(c.c23, rho_in), ux_in);
    const float a16 = __fmul_rn(__fmul_rn(c.c16, rho_in), ux_in);
    const float hy = __fmul_rn(__fmul_rn(0.5f, rho_in), uy_in);
    const float dy = __fmul_rn(0.5f, diff_y), dz = __fmul_rn(0.5f, diff_z);
    v[1] = __fadd_rn(v[2], a23);
    v[7] = __fsub_rn(__fadd_rn(__fadd_rn(v[10], a16), hy), dy);
    v[9] = __fadd_rn(__fsub_rn(__fadd_rn(v[8], a16), hy), dy);
    v[11] = __fsub_rn(__fadd_rn(v[14], a16), dz);
    v[13] = __fadd_rn(__fadd_rn(v[12], a16), dz);
}

// Gather the post-stream, post-boundary populations S(x, y, z) of the stored state.
// pull = false: the stored array already is a post-stream state (after initialisation or
// an import), read in place.
// RAW: return the stored values themselves (the deviations h = f - w of the shifted forms,
// for collide<.., DEV = true>); the Zou-He inlet is applied to f = h + w and shifted back.
// For float32 storage RAW changes nothing.
// IDX32: element indices in 32-bit unsigned arithmetic (valid while 19 * plane < 2^32),
// one wide multiply-add per address instead of 64-bit index arithmetic.
template <int S, bool PULL, bool RAW = false, bool IDX32 = false>
__device__ __forceinline__ void gather(const typename Pop<S>::T* __restrict__ f, const Grid& g,
                                       const Coef& c, int x, int y, int z, float (&v)[19]) {
    using P = Pop<S>;
    using I = typename std::conditional<IDX32, unsigned, long long>::type;
    constexpr bool kRaw = RAW && P::kShifted;
    const I plane = (I)g.plane;
    if (!PULL) {
        const I cell = ((I)z * (I)g.ny + (I)y) * (I)g.pitch + (I)x;
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const I e = (I)q * plane + cell;
            v[q] = !in_bounds((long long)e, 19LL * g.plane, g.status) ? 0.0f
                   : kRaw ? P::ld_raw(f + e) : P::ld(f + e, q);
        }
        return;
    }
    const int xe = (x == g.nx - 1) ? g.nx - 2 : x;  // outlet: copy of column Nx-2
    const int ym = (y == 0) ? g.ny - 1 : y - 1;
    const int yp = (y == g.ny - 1) ? 0 : y + 1;
    const int zm = (z == 0) ? g.nz - 1 : z - 1;
    const int zp = (z == g.nz - 1) ? 0 : z + 1;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const int sy = ey(q) == 1 ? ym : (ey(q) == -1 ? yp : y);
        const int sz = ez(q) == 1 ? zm : (ez(q) == -1 ? zp : z);
        const int sx = xe - ex(q);
        if (ex(q) == 1 && xe == 0) {
            v[q] = 0.0f;  // inlet unknown, rebuilt by Zou-He below
        } else {
            const I e = (I)q * plane + ((I)sz * (I)g.ny + (I)sy) * (I)g.pitch + (I)sx;
            v[q] = !in_bounds((long long)e, 19LL * g.plane, g.status) ? 0.0f
                   : kRaw ? P::ld_raw(f + e) : P::ld(f + e, q);
        }
    }
    if (xe == 0) {
        if (kRaw) {
#pragma unroll
            for (int q = 0; q < 19; ++q) v[q] += wq(q);
        }
        zou_he(v, c);
        if (kRaw) {
#pragma unroll
            for (int q = 0; q < 19; ++q) v[q] -= wq(q);
        }
    }
}

// Store a population vector produced by gather<.., RAW = true> + collide<.., DEV = kShifted>.
template <int S, bool IDX32 = false>
__device__ __forceinline__ void store_raw(typename Pop<S>::T* __restrict__ f, const Grid& g,
                                          long long cell, const float (&v)[19]) {
    using I = typename std::conditional<IDX32, unsigned, long long>::type;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const I e = (I)q * (I)g.plane + (I)cell;
        if (in_bounds((long long)e, 19LL * g.plane, g.status)) Pop<S>::st_raw(f + e, v[q]);
    }
}

// Zeroth, first and second raw moments of a population vector.
struct Moments {
    float rho, mx, my, mz, pxx, pyy, pzz, pxy, pxz, pyz;
};

__device__ __forceinline__ Moments moments(const float (&f)[19]) {
    Moments m;
    const float sx = f[1] + f[2], sy = f[3] + f[4], sz = f[5] + f[6];
    const float a = f[7] + f[8], b = f[9] + f[10], cc = f[11] + f[12], d = f[13] + f[14];
    const float e = f[15] + f[16], h = f[17] + f[18];
    m.rho = f[0] + (sx + sy + sz) + (a + b) + (cc + d) + (e + h);
    m.mx = (f[1] - f[2]) + (f[7] - f[8]) + (f[9] - f[10]) + (f[11] - f[12]) + (f[13] - f[14]);
    m.my = (f[3] - f[4]) + (a - b) + (f[15] - f[16]) + (f[17] - f[18]);
    m.mz = (f[5] - f[6]) + (cc - d) + (e - h);
    m.pxx = sx + (a + b) + (cc + d);
    m.pyy = sy + (a + b) + (e + h);
    m.pzz = sz + (cc + d) + (e + h);
    m.pxy = (f[7] + f[10]) - (f[8] + f[9]);
    m.pxz = (f[11] + f[14]) - (f[12] + f[13]);
    m.pyz = (f[15] + f[18]) - (f[16] + f[17]);
    return m;
}

// ---------------------------------------------------------------- collision arithmetic
// The collision is written once over a value type V:
//   F1  one float32 (one cell), plain operators: the compiler may contract a*b + c;
//   V1  one float32 with explicitly rounded operations (no contraction);
//   V2  two float32 lanes (two cells) evaluated by the packed f32x2 instructions of
//       sm_100-class GPUs, which halve the issue slots of the arithmetic.
// V1 and V2 perform the same IEEE round-to-nearest operations, so the 16-bit kernels that
// compute one cell (V1) or two cells (V2) per thread give identical bits. The float32
// kernels are bound by memory bandwidth and use F1.
struct F1 {
    float x;
};
struct V1 {
    float x;
};
struct V2 {
    unsigned long long x;
};

__device__ __forceinline__ F1 operator+(F1 a, F1 b) { return {a.x + b.x}; }
__device__ __forceinline__ F1 operator-(F1 a, F1 b) { return {a.x - b.x}; }
__device__ __forceinline__ F1 operator*(F1 a, F1 b) { return {a.x * b.x}; }
__device__ __forceinline__ F1 vfma(F1 a, F1 b, F1 c) { return {fmaf(a.x, b.x, c.x)}; }
__device__ __forceinline__ F1 vsplat(float a, F1) { return {a}; }
__device__ __forceinline__ F1 vrcp(F1 a) { return {__frcp_rn(a.x)}; }

__device__ __forceinline__ V1 operator+(V1 a, V1 b) { return {__fadd_rn(a.x, b.x)}; }
__device__ __forceinline__ V1 operator-(V1 a, V1 b) { return {__fsub_rn(a.x, b.x)}; }
__device__ __forceinline__ V1 operator*(V1 a, V1 b) { return {__fmul_rn(a.x, b.x)}; }
__device__ __forceinline__ V1 vfma(V1 a, V1 b, V1 c) { return {__fmaf_rn(a.x, b.x, c.x)}; }
__device__ __forceinline__ V1 vsplat(float a, V1) { return {a}; }
__device__ __forceinline__ V1 vrcp(V1 a) { return {__frcp_rn(a.x)}; }
__device__ __forceinline__ V1 vdiv(V1 a, V1 b) { return {__fdiv_rn(a.x, b.x)}; }
// x / 3 and x / 9, correctly rounded, without a division instruction sequence: the
// quotient RN(x * RN(1/d)) corrected once by its exact remainder (Markstein's iteration
// for division by a constant, P. Markstein, "IA-64 and Elementary Functions", 2000). For
// d = 3 and d = 9 it returns RN(x / d) for every float x with a normal or zero
// numerator (checked exhaustively against IEEE division over all positive normal x; the
// method is odd in x). It does not hold for every divisor, so it is used for these two.
template <int D>
__device__ __forceinline__ V1 vdiv_int(V1 x) {
    static_assert(D == 3 || D == 9, "exactness checked for 3 and 9 only");
    constexpr float d = (float)D, rd = 1.0f / (float)D;
    const float q0 = __fmul_rn(x.x, rd);
    const float rem = __fmaf_rn(-q0, d, x.x);
    return {__fmaf_rn(rem, rd, q0)};
}

__device__ __forceinline__ V2 operator+(V2 a, V2 b) {
    V2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.x) : "l"(a.x), "l"(b.x));
    return d;
}
__device__ __forceinline__ V2 operator-(V2 a, V2 b) {
    V2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.x) : "l"(a.x), "l"(b.x));
    return d;
}
__device__ __forceinline__ V2 operator*(V2 a, V2 b) {
    V2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d.x) : "l"(a.x), "l"(b.x));
    return d;
}
__device__ __forceinline__ V2 vfma(V2 a, V2 b, V2 c) {
    V2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.x) : "l"(a.x), "l"(b.x), "l"(c.x));
    return d;
}
__device__ __forceinline__ V2 vpack(float a, float b) {
    V2 d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d.x) : "f"(a), "f"(b));
    return d;
}
__device__ __forceinline__ float2 vunpack(V2 v) {
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v.x));
    return r;
}
__device__ __forceinline__ V2 vsplat(float a, V2) { return vpack(a, a); }
__device__ __forceinline__ V2 vrcp(V2 a) {
    const float2 t = vunpack(a);
    return vpack(__frcp_rn(t.x), __frcp_rn(t.y));
}

// Divergence monitor, the device form of main_moving.py:143-145 (which stops the run when
// rho_min < 0.3 or a field is not finite on its vis steps): every collision compares its
// cell's density with the floor; a density below it or not finite (NaN fails both tests)
// sets a sticky status bit that the host reads between steps or graph replays. Two
// comparisons per cell on a value the collision computes anyway; no extra memory traffic.
__device__ __forceinline__ void monitor_rho(const Coef& c, float r) {
    if (c.status && !(r >= c.rho_floor && r <= 3.0e38f)) atomicOr(c.status, kStatusDiverged);
}
__device__ __forceinline__ void monitor_rho(const Coef& c, F1 r) { monitor_rho(c, r.x); }
__device__ __forceinline__ void monitor_rho(const Coef& c, V1 r) { monitor_rho(c, r.x); }
__device__ __forceinline__ void monitor_rho(const Coef& c, V2 r) {
    const float2 t = vunpack(r);
    monitor_rho(c, t.x);
    monitor_rho(c, t.y);
}

// Cascaded collision in central-moment space followed by the raw-moment back transform,
// in place on f. (Fx, Fy, Fz) is the body-force density at the cell (zero gives the
// unforced result).
// DEV: f holds deviations h = f - w (shifted storage) on input and output. Moments of the
// weights are added to the zeroth and second moments (sum w = 1, sum w e_a e_b = d_ab / 3)
// and subtracted again from the raw post-collision moments before the back transform
// (sum w = 1, sum w e_a^2 = 1/3, sum w e_a^2 e_b^2 = 1/9; all other moments of w vanish),
// so no per-population shift is needed.
// HO: third- and fourth-order central moments do not relax fully to equilibrium; ho holds
// their post-collision values (k210, k120, k201, k021, k102, k012, then k220 - r/9,
// k202 - r/9, k022 - r/9), which the closure computes (the reference's s_q = s_pi = 1
// gives zeros).
// SVC: the deviatoric second-order moments relax with the per-cell rate s (osv_cell =
// 1 - s) instead of s_v (eddy-viscosity closure).
template <class V, bool FORCE, bool DEV, bool HO = false, bool SVC = false>
__device__ __forceinline__ void collide_v(V (&f)[19], const Coef& c, V Fx, V Fy, V Fz,
                                          const V* ho = nullptr, V osv_cell = V{}) {
    const V z0 = f[0];
    const V one = vsplat(1.0f, z0), third = vsplat(1.0f / 3.0f, z0);
    const V half = vsplat(0.5f, z0), quarter = vsplat(0.25f, z0), two = vsplat(2.0f, z0);
    const V m_two = vsplat(-2.0f, z0);
    // zeroth, first and second raw moments
    const V sx = f[1] + f[2], sy = f[3] + f[4], sz = f[5] + f[6];
    const V a = f[7] + f[8], b = f[9] + f[10], cc = f[11] + f[12], d = f[13] + f[14];
    const V e = f[15] + f[16], h = f[17] + f[18];
    const V ab = a + b, cd = cc + d, eh = e + h;
    const V drho = (((f[0] + ((sx + sy) + sz)) + ab) + cd) + eh;
    const V mx = ((((f[1] - f[2]) + (f[7] - f[8])) + (f[9] - f[10])) + (f[11] - f[12])) + (f[13] - f[14]);
    const V my = (((f[3] - f[4]) + (a - b)) + (f[15] - f[16])) + (f[17] - f[18]);
    const V mz = ((f[5] - f[6]) + (cc - d)) + (e - h);
    V pxx = (sx + ab) + cd, pyy = (sy + ab) + eh, pzz = (sz + cd) + eh;
    const V pxy = (f[7] + f[10]) - (f[8] + f[9]);
    const V pxz = (f[11] + f[14]) - (f[12] + f[13]);
    const V pyz = (f[15] + f[18]) - (f[16] + f[17]);
    V r = drho;
    if (DEV) {
        r = drho + one;
        pxx = pxx + third;
        pyy = pyy + third;
        pzz = pzz + third;
    }
    monitor_rho(c, r);
    const V inv = vrcp(r);
    V u = mx * inv, v = my * inv, w = mz * inv;
    if (FORCE) {
        u = vfma(half * Fx, inv, u);
        v = vfma(half * Fy, inv, v);
        w = vfma(half * Fz, inv, w);
    }
    const V ur = u * r, vr = v * r, wr = w * r;
    // second-order central moments about the shifted velocity
    const V k200 = vfma(u, vfma(m_two, mx, ur), pxx);
    const V k020 = vfma(v, vfma(m_two, my, vr), pyy);
    const V k002 = vfma(w, vfma(m_two, mz, wr), pzz);
    const V k110 = pxy - vfma(u, my - vr, v * mx);
    const V k101 = pxz - vfma(u, mz - wr, w * mx);
    const V k011 = pyz - vfma(v, mz - wr, w * my);
    // relaxation (clbm_moving.py:170-196)
    const V osv = SVC ? osv_cell : vsplat(c.one_m_sv, z0);
    const V k110s = k110 * osv, k101s = k101 * osv, k011s = k011 * osv;
    const V kA = (k200 + k020) + k002;
    const V kAs = vfma(vsplat(-c.s_e, z0), kA - r, kA);
    const V kDs = (k200 - k020) * osv, kEs = (k200 - k002) * osv;
    const V k200s = ((kAs + kDs) + kEs) * third;
    const V k020s = (vfma(m_two, kDs, kAs) + kEs) * third;
    const V k002s = vfma(m_two, kEs, kAs + kDs) * third;
    // fourth-order equilibrium r/9; its weight part 1/9 is removed here in the shifted form
    const V r9 = (DEV ? drho : r) * vsplat(1.0f / 9.0f, z0);
    // raw post-collision moments (third-order central moments relax to 0, fourth to r/9)
    const V uu = u * u, vv = v * v, ww = w * w;
    const V u2 = two * u, v2 = two * v, w2 = two * w;
    const V T110 = vfma(u, vr, k110s), T101 = vfma(u, wr, k101s), T011 = vfma(v, wr, k011s);
    V T200 = vfma(u, ur, k200s), T020 = vfma(v, vr, k020s), T002 = vfma(w, wr, k002s);
    const V T210 = vfma(u2, k110s, vfma(v, k200s, uu * vr));
    const V T120 = vfma(v2, k110s, vfma(u, k020s, vv * ur));
    const V T201 = vfma(u2, k101s, vfma(w, k200s, uu * wr));
    const V T021 = vfma(v2, k011s, vfma(w, k020s, vv * wr));
    const V T102 = vfma(w2, k101s, vfma(u, k002s, ww * ur));
    const V T012 = vfma(w2, k011s, vfma(v, k002s, ww * vr));
    V T220 = vfma(u2 * v2, k110s, vfma(vv, k200s, vfma(uu, k020s, vfma(uu, vv * r, r9))));
    V T202 = vfma(u2 * w2, k101s, vfma(ww, k200s, vfma(uu, k002s, vfma(uu, ww * r, r9))));
    V T022 = vfma(v2 * w2, k011s, vfma(ww, k020s, vfma(vv, k002s, vfma(vv, ww * r, r9))));
    V T210x = T210, T120x = T120, T201x = T201, T021x = T021, T102x = T102, T012x = T012;
    if (HO) {
        // binomial terms of the non-zero third/fourth-order post-collision central moments
        T210x = T210 + ho[0]; T120x = T120 + ho[1]; T201x = T201 + ho[2];
        T021x = T021 + ho[3]; T102x = T102 + ho[4]; T012x = T012 + ho[5];
        T220 = T220 + vfma(u2, ho[1], vfma(v2, ho[0], ho[6]));
        T202 = T202 + vfma(u2, ho[4], vfma(w2, ho[2], ho[7]));
        T022 = T022 + vfma(v2, ho[5], vfma(w2, ho[3], ho[8]));
    }
    if (DEV) {
        T200 = T200 - third;
        T020 = T020 - third;
        T002 = T002 - third;
    }
    // closed form of M_raw^-1 (config_moving.py:62-73)
    f[0] = ((DEV ? drho : r) - ((T200 + T020) + T002)) + ((T220 + T202) + T022);
    const V A1 = half * ((T200 - T220) - T202), B1 = half * ((ur - T120x) - T102x);
    const V A2 = half * ((T020 - T220) - T022), B2 = half * ((vr - T210x) - T012x);
    const V A3 = half * ((T002 - T202) - T022), B3 = half * ((wr - T201x) - T021x);
    f[1] = A1 + B1; f[2] = A1 - B1;
    f[3] = A2 + B2; f[4] = A2 - B2;
    f[5] = A3 + B3; f[6] = A3 - B3;
    // plane diagonals: f = (T_aabb + e_a e_b T_ab + e_b T_aab + e_a T_abb) / 4
    {
        const V sp = quarter * (T220 + T110), sm = quarter * (T220 - T110);
        const V pa = quarter * (T210x + T120x), ma = quarter * (T210x - T120x);
        f[7] = sp + pa;    // (+1,+1)
        f[8] = sm + ma;    // (-1,+1)
        f[9] = sm - ma;    // (+1,-1)
        f[10] = sp - pa;   // (-1,-1)
    }
    {
        const V sp = quarter * (T202 + T101), sm = quarter * (T202 - T101);
        const V pa = quarter * (T201x + T102x), ma = quarter * (T201x - T102x);
        f[11] = sp + pa;
        f[12] = sm + ma;
        f[13] = sm - ma;
        f[14] = sp - pa;
    }
    {
        const V sp = quarter * (T022 + T011), sm = quarter * (T022 - T011);
        const V pa = quarter * (T021x + T012x), ma = quarter * (T021x - T012x);
        f[15] = sp + pa;
        f[16] = sm + ma;
        f[17] = sm - ma;
        f[18] = sp - pa;
    }
    if (FORCE) {
        // Guo forcing: w_q (1 - s_v/2) [ (e - u)/cs2 + (e.u) e / cs2^2 ] . F
        const V three = vsplat(3.0f, z0), nine = vsplat(9.0f, z0);
        const V u3 = three * u, v3 = three * v, w3 = three * w;
        const V u9 = nine * u, v9 = nine * v, w9 = nine * w;
        // per population: 9 (e.u)(e.F) + 3 e.F - 3 u.F, with e_a in {-1, 0, 1}
        const V zero = vsplat(0.0f, z0);
        const V nuF3 = zero - vfma(u3, Fx, vfma(v3, Fy, w3 * Fz));
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            V eu9 = zero, eF = zero;
            if (ex(q) > 0) { eu9 = eu9 + u9; eF = eF + Fx; }
            if (ex(q) < 0) { eu9 = eu9 - u9; eF = eF - Fx; }
            if (ey(q) > 0) { eu9 = eu9 + v9; eF = eF + Fy; }
            if (ey(q) < 0) { eu9 = eu9 - v9; eF = eF - Fy; }
            if (ez(q) > 0) { eu9 = eu9 + w9; eF = eF + Fz; }
            if (ez(q) < 0) { eu9 = eu9 - w9; eF = eF - Fz; }
            const V term = vfma(eu9, eF, vfma(three, eF, nuF3));
            f[q] = vfma(vsplat(c.wc[q], z0), term, f[q]);
        }
    }
}

// Float32 storage: the collision in the reference's own operation order wherever that
// order is cheap to keep, every operation explicitly rounded (V1, no contraction):
//  * rho and the momentum as sums over q in q order, u = m / rho + (F / 2) / rho
//    (_macro_with_force, clbm_moving.py:105-115);
//  * the relaxation with its divisions by 3 and 9 (clbm_moving.py:170-196);
//  * the raw post-collision moments T term by term, left to right (clbm_moving.py:198-231;
//    the third-order central moments are zero there, and adding a zero is exact);
//  * the back transform f*_q = sum_j M_raw^-1[q][j] T_j summed over j in order
//    (clbm_moving.py:233-238). The entries of M_raw^-1 (config_moving.py:62-73) are 0,
//    +-1/4, +-1/2 and +-1: every product is exact and the zero terms add nothing, so the
//    91 non-zero terms summed in j order round exactly as the reference's dense 19 x 19 loop
//    does for the same T (a common factor 1/2 or 1/4 is applied after the sum, which scales
//    every rounding by that power of two).
// Keeping the back transform's summation order matters for mass: in a nearly uniform flow
// every cell rounds the same values the same way, so a summation order whose roundings do
// not cancel over the 19 populations shifts the total mass by the same amount in every cell
// and step.
// Unforced cells (nearly all of them) take the second-order central moments from the raw
// moments (pair sums, shifted by the velocity) instead of the reference's 19-term sums of
// f (e - u)^p, which would cost about 500 more operations per cell. Forced cells -- the
// IBM force box, a few per cent of the lattice, run by their own pass -- take the
// reference's sums and its Guo term too, so where the body acts the step repeats the
// reference's arithmetic operation for operation.
struct RefMacro {
    V1 r, mx, my, mz, u, v, w;
};

template <bool FORCE>
__device__ __forceinline__ RefMacro ref_macro(const V1 (&f)[19], const Coef& c, V1 Fx, V1 Fy,
                                              V1 Fz) {
    using V = V1;
    RefMacro m;
    // _macro_with_force: r += f_q, m += e_q f_q in q order (e_q f_q is +-f_q or an exact 0)
    V r = f[0];
#pragma unroll
    for (int q = 1; q < 19; ++q) r = r + f[q];
    monitor_rho(c, r);
    m.r = r;
    m.mx = ((((((((f[1] - f[2]) + f[7]) - f[8]) + f[9]) - f[10]) + f[11]) - f[12]) + f[13]) - f[14];
    m.my = ((((((((f[3] - f[4]) + f[7]) + f[8]) - f[9]) - f[10]) + f[15]) - f[16]) + f[17]) - f[18];
    m.mz = ((((((((f[5] - f[6]) + f[11]) + f[12]) - f[13]) - f[14]) + f[15]) + f[16]) - f[17]) - f[18];
    m.u = vdiv(m.mx, r);
    m.v = vdiv(m.my, r);
    m.w = vdiv(m.mz, r);
    if (FORCE) {
        const V half = vsplat(0.5f, r);
        m.u = m.u + vdiv(half * Fx, r);
        m.v = m.v + vdiv(half * Fy, r);
        m.w = m.w + vdiv(half * Fz, r);
    }
    return m;
}

// Relaxation, raw post-collision moments and back transform from the second-order
// central moments (clbm_moving.py:170-238); writes f.
__device__ __forceinline__ void ref_relax_back(V1 (&f)[19], const Coef& c, const RefMacro& m,
                                               V1 k200, V1 k020, V1 k002, V1 k110, V1 k101,
                                               V1 k011, V1 osv) {
    using V = V1;
    const V r = m.r, u = m.u, v = m.v, w = m.w;
    const V half = vsplat(0.5f, r), quarter = vsplat(0.25f, r), two = vsplat(2.0f, r);
    const V four = vsplat(4.0f, r);
    // cascade relaxation, clbm_moving.py:170-196
    const V k110s = k110 * osv, k101s = k101 * osv, k011s = k011 * osv;
    const V kA = (k200 + k020) + k002;
    const V kAs = kA - vsplat(c.s_e, r) * (kA - r);
    const V kDs = (k200 - k020) * osv, kEs = (k200 - k002) * osv;
    const V k200s = vdiv_int<3>((kAs + kDs) + kEs);
    const V k020s = vdiv_int<3>((kAs - two * kDs) + kEs);
    const V k002s = vdiv_int<3>((kAs + kDs) - two * kEs);
    const V r9 = vdiv_int<9>(r);
    // raw post-collision moments, clbm_moving.py:198-231
    const V ur = u * r, vr = v * r, wr = w * r;
    const V uu = u * u, vv = v * v, ww = w * w, uv = u * v, uw = u * w, vw = v * w;
    const V T110 = k110s + uv * r, T101 = k101s + uw * r, T011 = k011s + vw * r;
    const V T200 = k200s + uu * r, T020 = k020s + vv * r, T002 = k002s + ww * r;
    const V T210 = ((two * u) * k110s + v * k200s) + (uu * v) * r;
    const V T120 = ((two * v) * k110s + u * k020s) + (uv * v) * r;
    const V T201 = ((two * u) * k101s + w * k200s) + (uu * w) * r;
    const V T021 = ((two * v) * k011s + w * k020s) + (vv * w) * r;
    const V T102 = ((two * w) * k101s + u * k002s) + (uw * w) * r;
    const V T012 = ((two * w) * k011s + v * k002s) + (vw * w) * r;
    const V T220 = (((r9 + ((four * u) * v) * k110s) + vv * k200s) + uu * k020s) + ((uu * v) * v) * r;
    const V T202 = (((r9 + ((four * u) * w) * k101s) + ww * k200s) + uu * k002s) + ((uu * w) * w) * r;
    const V T022 = (((r9 + ((four * v) * w) * k011s) + ww * k020s) + vv * k002s) + ((vv * w) * w) * r;
    // back transform: non-zero terms of each row of M_raw^-1 in column order
    f[0] = (((((r - T200) - T020) - T002) + T220) + T202) + T022;
    f[1] = half * ((((((ur + T200) - T120) - T102) - T220) - T202));
    f[2] = half * ((((((T200 - ur) + T120) + T102) - T220) - T202));
    f[3] = half * ((((((vr + T020) - T210) - T012) - T220) - T022));
    f[4] = half * ((((((T020 - vr) + T210) + T012) - T220) - T022));
    f[5] = half * ((((((wr + T002) - T201) - T021) - T202) - T022));
    f[6] = half * ((((((T002 - wr) + T201) + T021) - T202) - T022));
    f[7] = quarter * (((T110 + T210) + T120) + T220);
    f[8] = quarter * (((T210 - T110) - T120) + T220);
    f[9] = quarter * ((T120 - (T110 + T210)) + T220);
    f[10] = quarter * (((T110 - T210) - T120) + T220);
    f[11] = quarter * (((T101 + T201) + T102) + T202);
    f[12] = quarter * (((T201 - T101) - T102) + T202);
    f[13] = quarter * ((T102 - (T101 + T201)) + T202);
    f[14] = quarter * (((T101 - T201) - T102) + T202);
    f[15] = quarter * (((T011 + T021) + T012) + T022);
    f[16] = quarter * (((T021 - T011) - T012) + T022);
    f[17] = quarter * ((T012 - (T011 + T021)) + T022);
    f[18] = quarter * (((T011 - T021) - T012) + T022);
}

// Unforced float32 collision (the bulk of the lattice).
template <bool SVC = false>
__device__ __forceinline__ void collide_ref(V1 (&f)[19], const Coef& c, V1 osv_cell = V1{}) {
    using V = V1;
    const V zero = vsplat(0.0f, f[0]), m_two = vsplat(-2.0f, f[0]);
    const RefMacro m = ref_macro<false>(f, c, zero, zero, zero);
    const V r = m.r, u = m.u, v = m.v, w = m.w;
    // second-order raw moments from pair sums, central moments about u
    const V sx = f[1] + f[2], sy = f[3] + f[4], sz = f[5] + f[6];
    const V a = f[7] + f[8], b = f[9] + f[10], cc = f[11] + f[12], d = f[13] + f[14];
    const V e = f[15] + f[16], h = f[17] + f[18];
    const V ab = a + b, cd = cc + d, eh = e + h;
    const V pxx = (sx + ab) + cd, pyy = (sy + ab) + eh, pzz = (sz + cd) + eh;
    const V pxy = (f[7] + f[10]) - (f[8] + f[9]);
    const V pxz = (f[11] + f[14]) - (f[12] + f[13]);
    const V pyz = (f[15] + f[18]) - (f[16] + f[17]);
    const V ur = u * r, vr = v * r, wr = w * r;
    const V k200 = vfma(u, vfma(m_two, m.mx, ur), pxx);
    const V k020 = vfma(v, vfma(m_two, m.my, vr), pyy);
    const V k002 = vfma(w, vfma(m_two, m.mz, wr), pzz);
    const V k110 = pxy - vfma(u, m.my - vr, v * m.mx);
    const V k101 = pxz - vfma(u, m.mz - wr, w * m.mx);
    const V k011 = pyz - vfma(v, m.mz - wr, w * m.my);
    const V osv = SVC ? osv_cell : vsplat(c.one_m_sv, r);
    ref_relax_back(f, c, m, k200, k020, k002, k110, k101, k011, osv);
}

// Forced float32 collision: _macro_with_force, the central moments as the reference's sums
// over q of f_q (e_q - u)^p (clbm_moving.py:139-168), relaxation and back transform as
// above, and the Guo term as the reference writes it (clbm_moving.py:240-249):
// f*_q += (w_q (1 - s_v / 2)) [((e - u) / cs2 + (e.u) e / cs2^2) . F], with the float32
// constants cs2 = 1/3 and cs2^2. (e_a - u_a) / cs2 takes three values per axis and
// (e.u) e_a / cs2^2 is +-(e.u) / cs2^2 or an exact zero, with (e.u) of opposite directions
// exact negatives, so 18 divisions give every quotient the reference forms.
__device__ __forceinline__ void collide_ref_forced(V1 (&f)[19], const Coef& c, V1 Fx, V1 Fy,
                                                   V1 Fz) {
    using V = V1;
    const V zero = vsplat(0.0f, f[0]);
    const RefMacro m = ref_macro<true>(f, c, Fx, Fy, Fz);
    const V u = m.u, v = m.v, w = m.w;
    V k110 = zero, k101 = zero, k011 = zero, k200 = zero, k020 = zero, k002 = zero;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const V xix = vsplat((float)ex(q), zero) - u;
        const V xiy = vsplat((float)ey(q), zero) - v;
        const V xiz = vsplat((float)ez(q), zero) - w;
        const V fx_ = f[q] * xix, fy_ = f[q] * xiy;
        k110 = k110 + fx_ * xiy;
        k101 = k101 + fx_ * xiz;
        k011 = k011 + fy_ * xiz;
        k200 = k200 + f[q] * (xix * xix);
        k020 = k020 + f[q] * (xiy * xiy);
        k002 = k002 + f[q] * (xiz * xiz);
    }
    ref_relax_back(f, c, m, k200, k020, k002, k110, k101, k011, vsplat(c.one_m_sv, zero));
    const V cs2 = vsplat(1.0f / 3.0f, zero);
    const V cs4 = vsplat((float)((1.0 / 3.0) * (1.0 / 3.0)), zero);
    const V one = vsplat(1.0f, zero);
    // (e_a - u_a) / cs2 for e_a = -1, 0, +1
    const V Ax[3] = {vdiv(zero - one - u, cs2), vdiv(zero - u, cs2), vdiv(one - u, cs2)};
    const V Ay[3] = {vdiv(zero - one - v, cs2), vdiv(zero - v, cs2), vdiv(one - v, cs2)};
    const V Az[3] = {vdiv(zero - one - w, cs2), vdiv(zero - w, cs2), vdiv(one - w, cs2)};
    // (e.u) / cs2^2 of the first direction of each opposite pair (clbm_moving.py order
    // x, y, z within e.u); the opposite direction takes its negative
    V D[19];
    D[0] = zero;
#pragma unroll
    for (int q = 1; q < 19; ++q) {
        if (opposite(q) < q) {
            D[q] = zero - D[opposite(q)];
            continue;
        }
        V eu = zero;
        bool first = true;
        if (ex(q) != 0) { eu = ex(q) > 0 ? u : zero - u; first = false; }
        if (ey(q) != 0) { const V t = ey(q) > 0 ? v : zero - v; eu = first ? t : eu + t; first = false; }
        if (ez(q) != 0) { const V t = ez(q) > 0 ? w : zero - w; eu = first ? t : eu + t; first = false; }
        D[q] = vdiv(eu, cs4);
    }
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const V cx = ex(q) == 0 ? Ax[1] : (ex(q) > 0 ? Ax[2] + D[q] : Ax[0] - D[q]);
        const V cy = ey(q) == 0 ? Ay[1] : (ey(q) > 0 ? Ay[2] + D[q] : Ay[0] - D[q]);
        const V cz = ez(q) == 0 ? Az[1] : (ez(q) > 0 ? Az[2] + D[q] : Az[0] - D[q]);
        f[q] = f[q] + vsplat(c.wc[q], zero) * ((cx * Fx + cy * Fy) + cz * Fz);
    }
}

// Scalar entry point: one cell held as float[19]; float32 storage collides in the
// reference's order (collide_ref), the shifted 16-bit forms on the deviations (V1, the
// same rounded operations as the packed two-cell form).
template <bool FORCE, bool DEV = false>
__device__ __forceinline__ void collide(float (&f)[19], const Coef& c, float Fx, float Fy,
                                        float Fz) {
    V1 t[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) t[q].x = f[q];
    if (DEV) collide_v<V1, FORCE, true>(t, c, V1{Fx}, V1{Fy}, V1{Fz});
    else if (FORCE) collide_ref_forced(t, c, V1{Fx}, V1{Fy}, V1{Fz});
    else collide_ref(t, c);
#pragma unroll
    for (int q = 0; q < 19; ++q) f[q] = t[q].x;
}

// One cell with third- and fourth-order post-collision central moments given (closure).
template <bool DEV>
__device__ __forceinline__ void collide_ho(float (&f)[19], const Coef& c, const float (&ho)[9]) {
    using V = typename std::conditional<DEV, V1, F1>::type;
    V t[19], h[9];
#pragma unroll
    for (int q = 0; q < 19; ++q) t[q].x = f[q];
#pragma unroll
    for (int i = 0; i < 9; ++i) h[i].x = ho[i];
    collide_v<V, false, DEV, true>(t, c, V{0.f}, V{0.f}, V{0.f}, h);
#pragma unroll
    for (int q = 0; q < 19; ++q) f[q] = t[q].x;
}

// One cell whose deviatoric second-order moments relax with 1 - osv (closure).
template <bool DEV>
__device__ __forceinline__ void collide_sv(float (&f)[19], const Coef& c, float osv) {
    V1 t[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) t[q].x = f[q];
    if (DEV) collide_v<V1, false, true, false, true>(t, c, V1{0.f}, V1{0.f}, V1{0.f}, nullptr, V1{osv});
    else collide_ref<true>(t, c, V1{osv});
#pragma unroll
    for (int q = 0; q < 19; ++q) f[q] = t[q].x;
}

// Two cells at once with the packed arithmetic (same bits as two scalar calls).
template <bool FORCE, bool DEV>
__device__ __forceinline__ void collide2(float (&f0)[19], float (&f1)[19], const Coef& c,
                                         float F0x, float F0y, float F0z, float F1x, float F1y,
                                         float F1z) {
    V2 t[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) t[q] = vpack(f0[q], f1[q]);
    collide_v<V2, FORCE, DEV>(t, c, vpack(F0x, F1x), vpack(F0y, F1y), vpack(F0z, F1z));
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const float2 p = vunpack(t[q]);
        f0[q] = p.x;
        f1[q] = p.y;
    }
}

// Collision of the two cells of a thread. Shifted 16-bit forms (DEV): packed (f32x2) when
// both are computed, a zero force on the unforced lane when only one is forced (same
// values as the unforced path). Float32: one scalar call per cell.
template <bool DEV>
__device__ __forceinline__ void collide_pair(float (&h0)[19], float (&h1)[19], const Coef& c,
                                             bool use0, bool use1, bool frc0, bool frc1,
                                             float F0x, float F0y, float F0z, float F1x,
                                             float F1y, float F1z) {
    if (DEV && use0 && use1) {
        if (frc0 || frc1) collide2<true, DEV>(h0, h1, c, F0x, F0y, F0z, F1x, F1y, F1z);
        else collide2<false, DEV>(h0, h1, c, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f);
        return;
    }
    if (use0) {
        if (frc0) collide<true, DEV>(h0, c, F0x, F0y, F0z);
        else collide<false, DEV>(h0, c, 0.f, 0.f, 0.f);
    }
    if (use1) {
        if (frc1) collide<true, DEV>(h1, c, F1x, F1y, F1z);
        else collide<false, DEV>(h1, c, 0.f, 0.f, 0.f);
    }
}

// ------------------------------------------------------------------ 16-bit pair kernel
// Shifted 16-bit storage moves half the bytes of float32, so the one-cell kernel becomes
// issue-bound. This variant gives each thread two neighbouring cells (x0, x0 + 1), x0 even:
// every population is one aligned 32-bit load/store of a half2 (or bf16x2); the x-shifted
// pulls take the neighbour element from the adjacent lane with a warp shuffle (the lanes at
// the two warp edges load that one element themselves); the collision works on the
// deviations directly (collide<.., DEV = true>), both cells at once in packed f32x2.
template <int S> struct Pair;
template <> struct Pair<CLBM_STORE_F16S> {
    using T = __half;
    static __device__ __forceinline__ float2 ld2(const T* p) {
        return __half22float2(__ldg(reinterpret_cast<const __half2*>(p)));
    }
    static __device__ __forceinline__ float ld1(const T* p) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ void st2(T* p, float a, float b) {
        const __half2 h = __floats2half2_rn(a, b);
        *reinterpret_cast<unsigned int*>(p) = *reinterpret_cast<const unsigned int*>(&h);
    }
    static __device__ __forceinline__ void st1(T* p, float a) {
        *reinterpret_cast<unsigned short*>(p) = __half_as_ushort(__float2half_rn(a));
    }
};
template <> struct Pair<CLBM_STORE_BF16S> {
    using T = __nv_bfloat16;
    static __device__ __forceinline__ float2 ld2(const T* p) {
        return __bfloat1622float2(__ldg(reinterpret_cast<const __nv_bfloat162*>(p)));
    }
    static __device__ __forceinline__ float ld1(const T* p) { return __bfloat162float(__ldg(p)); }
    static __device__ __forceinline__ void st2(T* p, float a, float b) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        *reinterpret_cast<unsigned int*>(p) = *reinterpret_cast<const unsigned int*>(&h);
    }
    static __device__ __forceinline__ void st1(T* p, float a) {
        *reinterpret_cast<unsigned short*>(p) = __bfloat16_as_ushort(__float2bfloat16_rn(a));
    }
};

// Boundary columns of a pulled cell pair (x0, x0 + 1) of row (y, z), x0 even: the Zou-He
// inlet at x0 = 0 on f = h + w (clbm_moving.py:266-294) and the outlet column Nx-1, a copy
// of column Nx-2 (clbm_moving.py:296-300). For odd Nx the outlet is the first cell of the
// last pair and its populations are pulled again like column Nx-2's.
template <int S, bool IDX32, class P = Pair<S>>
__device__ __forceinline__ void pair_boundaries(const typename Pair<S>::T* __restrict__ fin,
                                                const Grid& g, const Coef& c, int x0, int y, int z,
                                                float (&h0)[19], float (&h1)[19]) {
    using I = typename std::conditional<IDX32, unsigned, long long>::type;
    if (x0 == 0) {
#pragma unroll
        for (int q = 0; q < 19; ++q) h0[q] += wq(q);
        zou_he(h0, c);
#pragma unroll
        for (int q = 0; q < 19; ++q) h0[q] -= wq(q);
    }
    if (x0 + 1 == g.nx - 1) {
#pragma unroll
        for (int q = 0; q < 19; ++q) h1[q] = h0[q];
    } else if (x0 == g.nx - 1) {
        const int ym = (y == 0) ? g.ny - 1 : y - 1;
        const int yp = (y == g.ny - 1) ? 0 : y + 1;
        const int zm = (z == 0) ? g.nz - 1 : z - 1;
        const int zp = (z == g.nz - 1) ? 0 : z + 1;
        const int xe = g.nx - 2;
        const I plane = (I)g.plane;
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const int sy = ey(q) == 1 ? ym : (ey(q) == -1 ? yp : y);
            const int sz = ez(q) == 1 ? zm : (ez(q) == -1 ? zp : z);
            const I e = (I)q * plane + ((I)sz * (I)g.ny + (I)sy) * (I)g.pitch + (I)(xe - ex(q));
            h0[q] = in_bounds((long long)e, 19LL * g.plane, g.status) ? P::ld1(fin + e) : 0.0f;
        }
    }
}

// Everything of a cell pair after its post-stream populations (h0, h1) are gathered: the
// force-box test, the body force per FMODE, the collision and the stores. act0 / act1: the
// cell lies inside the lattice. kForceOnlyBand (box pass): only the cells inside the force
// box are collided and stored; with ks, their clipped forces in units of 2^-40 are added to
// ks[0], ks[1] (exact).
template <int S, int FMODE, bool IDX32, class P = Pair<S>>
__device__ __forceinline__ void pair_finish(typename Pair<S>::T* __restrict__ fout, const Grid& g,
                                            const Coef& c, const ForceArgs& fa, int x0, int y, int z,
                                            bool act0, bool act1, float (&h0)[19], float (&h1)[19],
                                            long long* ks) {
    using I = typename std::conditional<IDX32, unsigned, long long>::type;
    const I plane = (I)g.plane;
    const I row = ((I)z * (I)g.ny + (I)y) * (I)g.pitch;
    // cells of the IBM force box: tested after the loads, so the box read does not delay them
    bool in0 = false, in1 = false;
    if (FMODE == kForceSkipBand || FMODE == kForceBand || FMODE == kForceOnlyBand) {
        const Band b = load_band(fa.dev, fa.slot);
        // the two cells share their row: the y/z part of the test once, then x per cell
        int oy = y - b.j0; if (oy < 0) oy += g.ny;
        int oz = z - b.k0; if (oz < 0) oz += g.nz;
        if (oy < b.jlen && oz < b.klen) {
            in0 = act0 && (unsigned)(x0 - b.i0) < (unsigned)b.ilen;
            in1 = act1 && (unsigned)(x0 + 1 - b.i0) < (unsigned)b.ilen;
        }
    }
    const bool use0 = act0 && (FMODE == kForceOnlyBand ? in0 : !(FMODE == kForceSkipBand && in0));
    const bool use1 = act1 && (FMODE == kForceOnlyBand ? in1 : !(FMODE == kForceSkipBand && in1));
    if (!use0 && !use1) return;
    // body force per cell
    float F0x = 0.f, F0y = 0.f, F0z = 0.f, F1x = 0.f, F1y = 0.f, F1z = 0.f;
    bool frc0 = false, frc1 = false;
    if (FMODE == kForceBand || FMODE == kForceOnlyBand) {
        frc0 = in0;
        frc1 = in1;
        if (in0 && in_bounds((long long)(row + x0), g.plane, g.status)) {
            F0x = fminf(fmaxf(qforce(fa.qx[row + x0]), -0.05f), 0.05f);
            F0y = fminf(fmaxf(qforce(fa.qy[row + x0]), -0.05f), 0.05f);
        }
        if (in1 && in_bounds((long long)(row + x0 + 1), g.plane, g.status)) {
            F1x = fminf(fmaxf(qforce(fa.qx[row + x0 + 1]), -0.05f), 0.05f);
            F1y = fminf(fmaxf(qforce(fa.qy[row + x0 + 1]), -0.05f), 0.05f);
        }
        if (FMODE == kForceOnlyBand && ks) {
            ks[0] += (long long)(F0x * kForceScale) + (long long)(F1x * kForceScale);
            ks[1] += (long long)(F0y * kForceScale) + (long long)(F1y * kForceScale);
        }
    } else if (FMODE == kForceDense) {
        frc0 = act0;
        frc1 = act1;
        if (act0) {
            F0x = fa.fx[row + x0]; F0y = fa.fy[row + x0]; F0z = fa.fz ? fa.fz[row + x0] : 0.f;
        }
        if (act1) {
            F1x = fa.fx[row + x0 + 1]; F1y = fa.fy[row + x0 + 1];
            F1z = fa.fz ? fa.fz[row + x0 + 1] : 0.f;
        }
    }
    collide_pair<true>(h0, h1, c, use0, use1, frc0, frc1, F0x, F0y, F0z, F1x, F1y, F1z);
    const long long nel = 19LL * g.plane;
    if (use0 && use1) {
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const I e = (I)q * plane + row + (I)x0;
            if (in_bounds((long long)e + 1, nel, g.status)) P::st2(fout + e, h0[q], h1[q]);
        }
    } else {
        if (use0) {
#pragma unroll
            for (int q = 0; q < 19; ++q) {
                const I e = (I)q * plane + row + (I)x0;
                if (in_bounds((long long)e, nel, g.status)) P::st1(fout + e, h0[q]);
            }
        }
        if (use1) {
#pragma unroll
            for (int q = 0; q < 19; ++q) {
                const I e = (I)q * plane + row + (I)x0 + 1;
                if (in_bounds((long long)e, nel, g.status)) P::st1(fout + e, h1[q]);
            }
        }
    }
}

// Cells (x0, x0 + 1) of row (y, z), x0 even, for a warp of consecutive pairs of one row
// (lanes past the lattice edge take part in the shuffles and store nothing).
// IDX32: element indices in 32-bit unsigned arithmetic (valid while 19 * plane < 2^32).
// P: the loads and stores of the storage form (Pair<S>).
// ks: force sums of the box pass (pair_finish).
template <int S, bool PULL, int FMODE, bool IDX32 = false, class P = Pair<S>>
__device__ __forceinline__ void pair_body(const typename Pair<S>::T* __restrict__ fin,
                                          typename Pair<S>::T* __restrict__ fout, const Grid& g,
                                          const Coef& c, const ForceArgs& fa, int x0, int y, int z,
                                          long long* ks = nullptr) {
    using I = typename std::conditional<IDX32, unsigned, long long>::type;
    const I plane = (I)g.plane;
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const bool act0 = x0 < g.nx, act1 = x0 + 1 < g.nx;
    // warp-uniform exit: every lane of a warp that stays takes part in the shuffles
    if (__all_sync(kFull, !act0)) return;
    const int x0c = min(x0, g.pitch - 2);  // in-row address for lanes past the lattice edge
    const I row = ((I)z * (I)g.ny + (I)y) * (I)g.pitch;
    float h0[19], h1[19];
    if (!PULL) {
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const I e = (I)q * plane + row + (I)x0c;
            const float2 p = in_bounds((long long)e + 1, 19LL * g.plane, g.status) ? P::ld2(fin + e)
                                                                                  : make_float2(0.f, 0.f);
            h0[q] = p.x;
            h1[q] = p.y;
        }
    } else {
        const int ym = (y == 0) ? g.ny - 1 : y - 1;
        const int yp = (y == g.ny - 1) ? 0 : y + 1;
        const int zm = (z == 0) ? g.nz - 1 : z - 1;
        const int zp = (z == g.nz - 1) ? 0 : z + 1;
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const int sy = ey(q) == 1 ? ym : (ey(q) == -1 ? yp : y);
            const int sz = ez(q) == 1 ? zm : (ez(q) == -1 ? zp : z);
            const I rb = (I)q * plane + ((I)sz * (I)g.ny + (I)sy) * (I)g.pitch;
            const typename P::T* rp = fin + rb;
            const float2 p = in_bounds((long long)(rb + (I)x0c) + 1, 19LL * g.plane, g.status)
                                 ? P::ld2(rp + x0c) : make_float2(0.f, 0.f);
            if (ex(q) == 0) {
                h0[q] = p.x;
                h1[q] = p.y;
            } else if (ex(q) == 1) {  // pull from x - 1
                float up = __shfl_up_sync(kFull, p.y, 1);
                if (lane == 0)
                    up = (x0 >= 1 && x0 - 1 < g.nx && in_bounds((long long)(rb + (I)(x0 - 1)), 19LL * g.plane, g.status))
                             ? P::ld1(rp + (x0 - 1)) : 0.0f;
                h0[q] = up;   // at x0 = 0 an inlet unknown, rebuilt by Zou-He below
                h1[q] = p.x;
            } else {                  // pull from x + 1
                float dn = __shfl_down_sync(kFull, p.x, 1);
                if (lane == 31)
                    dn = (x0 + 2 < g.nx && in_bounds((long long)(rb + (I)(x0 + 2)), 19LL * g.plane, g.status))
                             ? P::ld1(rp + (x0 + 2)) : 0.0f;
                h0[q] = p.y;
                h1[q] = dn;
            }
        }
        pair_boundaries<S, IDX32, P>(fin, g, c, x0, y, z, h0, h1);
    }
    pair_finish<S, FMODE, IDX32, P>(fout, g, c, fa, x0, y, z, act0, act1, h0, h1, ks);
}


// One cell of the full-grid pass: gather, force (per FMODE), collide, store.
// kForceOnlyBand (box pass): only a cell inside the force box is collided and stored; with
// ks, its clipped force in units of 2^-40 is added to ks[0], ks[1] (exact).
// IDX32: element indices in 32-bit unsigned arithmetic (valid while 19 * plane < 2^32).
template <int S, bool PULL, int FMODE, bool IDX32 = false>
__device__ __forceinline__ void stream_collide_cell(const typename Pop<S>::T* __restrict__ fin,
                                                    typename Pop<S>::T* __restrict__ fout,
                                                    const Grid& g, const Coef& c,
                                                    const ForceArgs& fa, int x, int y, int z,
                                                    long long* ks = nullptr) {
    // shifted storage: the collision works on the deviations (no per-population shift)
    constexpr bool DEV = Pop<S>::kShifted;
    float f[19];
    gather<S, PULL, true, IDX32>(fin, g, c, x, y, z, f);
    if (FMODE == kForceSkipBand) {
        // bulk pass of an IBM step: the cells of the force box are done by the box pass.
        // Tested after the gather, so the box read does not delay the population loads.
        const Band b = load_band(fa.dev, fa.slot);
        if (in_band(b, x, y, z, g.ny, g.nz)) return;
    }
    const long long cell = ((long long)z * g.ny + y) * g.pitch + x;
    if (FMODE == kForceNone || FMODE == kForceSkipBand) {
        collide<false, DEV>(f, c, 0.f, 0.f, 0.f);
    } else if (FMODE == kForceDense) {
        const bool ok = in_bounds(cell, g.plane, g.status);
        const float Fz = (fa.fz && ok) ? fa.fz[cell] : 0.0f;
        collide<true, DEV>(f, c, ok ? fa.fx[cell] : 0.0f, ok ? fa.fy[cell] : 0.0f, Fz);
    } else {
        const Band b = load_band(fa.dev, fa.slot);
        if (in_band(b, x, y, z, g.ny, g.nz)) {
            // Eulerian clip of _clip_forces (airfoil_moving.py:219-225) applied on read;
            // fz is always zero there.
            const bool ok = in_bounds(cell, g.plane, g.status);
            const float Fx = ok ? fminf(fmaxf(qforce(fa.qx[cell]), -0.05f), 0.05f) : 0.0f;
            const float Fy = ok ? fminf(fmaxf(qforce(fa.qy[cell]), -0.05f), 0.05f) : 0.0f;
            if (FMODE == kForceOnlyBand && ks) {
                ks[0] += (long long)(Fx * kForceScale);
                ks[1] += (long long)(Fy * kForceScale);
            }
            collide<true, DEV>(f, c, Fx, Fy, 0.0f);
        } else {
            if (FMODE == kForceOnlyBand) return;
            collide<false, DEV>(f, c, 0.f, 0.f, 0.f);
        }
    }
    store_raw<S, IDX32>(fout, g, cell, f);
}

// Forced stream-collide of box cell t of band b (the box pass, one cell). SUMS: also add
// the cell's clipped force, in units of 2^-40, to kx, ky (the Eulerian part of the
// lift/drag sums; every clipped value is an integer multiple of 2^-40, so the integer sums
// are exact in any order).
template <int S, bool PULL, bool SUMS = false>
__device__ __forceinline__ void box_pass_cell(const typename Pop<S>::T* __restrict__ fin,
                                              typename Pop<S>::T* __restrict__ fout,
                                              const Grid& g, const Coef& c, const ForceArgs& fa,
                                              const Band& b, int t, long long* kx = nullptr,
                                              long long* ky = nullptr) {
    int x, y, z;
    box_cell(b, g.ny, g.nz, t, x, y, z);
    float f[19];
    gather<S, PULL, true>(fin, g, c, x, y, z, f);
    const long long cell = ((long long)z * g.ny + y) * g.pitch + x;
    const bool ok = in_bounds(cell, g.plane, g.status);
    const float Fx = ok ? fminf(fmaxf(qforce(fa.qx[cell]), -0.05f), 0.05f) : 0.0f;
    const float Fy = ok ? fminf(fmaxf(qforce(fa.qy[cell]), -0.05f), 0.05f) : 0.0f;
    if (SUMS) {
        *kx += (long long)(Fx * kForceScale);
        *ky += (long long)(Fy * kForceScale);
    }
    collide<true, Pop<S>::kShifted>(f, c, Fx, Fy, 0.0f);
    store_raw<S>(fout, g, cell, f);
}

// Forced stream-collide of the cells of the IBM force box; block bx of nbx (blockDim.x threads)
// takes cells bx * blockDim.x + threadIdx.x, stepping by nbx * blockDim.x.
template <int S, bool PULL>
__device__ __forceinline__ void box_pass_body(const typename Pop<S>::T* __restrict__ fin,
                                              typename Pop<S>::T* __restrict__ fout,
                                              const Grid& g, const Coef& c, const ForceArgs& fa,
                                              int bx, int nbx) {
    const Band b = load_band(fa.dev, fa.slot);
    const int cells = b.ilen * b.jlen * b.klen;
    for (int t = bx * blockDim.x + threadIdx.x; t < cells; t += nbx * blockDim.x)
        box_pass_cell<S, PULL>(fin, fout, g, c, fa, b, t);
}

// The two pieces of band-prepare for one cell: zero the force of box cell t of band ob,
// and _macro_post (clbm_moving.py:305-321) of box cell t of band nb.
__device__ __forceinline__ void band_zero_cell(const Grid& g, long long* fx, long long* fy,
                                               const Band& ob, int t) {
    int x, y, z;
    box_cell(ob, g.ny, g.nz, t, x, y, z);
    const long long cell = ((long long)z * g.ny + y) * g.pitch + x;
    if (!in_bounds(cell, g.plane, g.status)) return;
    fx[cell] = 0;
    fy[cell] = 0;
}

template <int S, bool PULL>
__device__ __forceinline__ void band_macro_cell(const typename Pop<S>::T* __restrict__ fin,
                                                const Grid& g, const Coef& c, float* rho, float* ux,
                                                float* uy, float* uz, const Band& nb, int t) {
    int x, y, z;
    box_cell(nb, g.ny, g.nz, t, x, y, z);
    float f[19];
    gather<S, PULL>(fin, g, c, x, y, z, f);
    float r = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        r += f[q];
        mx += (float)ex(q) * f[q];
        my += (float)ey(q) * f[q];
        mz += (float)ez(q) * f[q];
    }
    const long long cell = ((long long)z * g.ny + y) * g.pitch + x;
    if (!in_bounds(cell, g.plane, g.status)) return;
    rho[cell] = r;
    ux[cell] = mx / r;
    uy[cell] = my / r;
    uz[cell] = mz / r;
}

// Zero the force box of the previous compute_force call (_zero_forces,
// airfoil_moving.py:132-137, restricted to where forces can be non-zero) and compute
// _macro_post (clbm_moving.py:305-321) of the current state on the box of this call.
template <int S, bool PULL>
__device__ __forceinline__ void band_prepare_body(const typename Pop<S>::T* __restrict__ fin,
                                                  const Grid& g, const Coef& c, IbmDev* dev,
                                                  long long* fx, long long* fy, float* rho,
                                                  float* ux, float* uy, float* uz,
                                                  bool compute_macro, int bx, int nbx) {
    // Box of this compute_force call (slot s & 1) and of the previous one (slot (s-1) & 1).
    const long long s = dev->step + 1;
    const Band nb = load_band(dev, (int)(s & 1));
    const Band ob = load_band(dev, (int)((s - 1) & 1));
    const int stride = nbx * blockDim.x;
    const int ocells = ob.ilen * ob.jlen * ob.klen;
    for (int t = bx * blockDim.x + threadIdx.x; t < ocells; t += stride) band_zero_cell(g, fx, fy, ob, t);
    if (!compute_macro) return;
    const int ncells = nb.ilen * nb.jlen * nb.klen;
    for (int t = bx * blockDim.x + threadIdx.x; t < ncells; t += stride)
        band_macro_cell<S, PULL>(fin, g, c, rho, ux, uy, uz, nb, t);
}

}  // namespace clbm
