// lbm_device.cuh -- device functions of the stream-collide pass shared by the
// single-lattice kernels (lbm_kernels.cu) and the batched ensemble kernels (ensemble.cu).
#pragma once

#include "clbm_internal.cuh"

namespace clbm {

// 3D Zou-He velocity inlet on the post-stream populations of an x = 0 cell,
// clbm_moving.py:266-294 (same operation order).
__device__ __forceinline__ void zou_he(float (&v)[19], const Coef& c) {
    const float ux_in = c.ux_in, uy_in = c.uy_in;
    float S_known = v[0] + v[3] + v[4] + v[5] + v[6] + v[15] + v[16] + v[17] + v[18];
    float S_out = v[2] + v[8] + v[10] + v[12] + v[14];
    float rho_in = (S_known + 2.0f * S_out) / (1.0f - ux_in);
    float diff_y = v[3] - v[4];
    float diff_z = v[5] - v[6];
    v[1] = v[2] + c.c23 * rho_in * ux_in;
    v[7] = v[10] + c.c16 * rho_in * ux_in + 0.5f * rho_in * uy_in - 0.5f * diff_y;
    v[9] = v[8] + c.c16 * rho_in * ux_in - 0.5f * rho_in * uy_in + 0.5f * diff_y;
    v[11] = v[14] + c.c16 * rho_in * ux_in - 0.5f * diff_z;
    v[13] = v[12] + c.c16 * rho_in * ux_in + 0.5f * diff_z;
}

// Gather the post-stream, post-boundary populations S(x, y, z) of the stored state.
// pull = false: the stored array already is a post-stream state (after initialisation or
// an import), read in place.
// RAW: return the stored values themselves (the deviations h = f - w of the shifted forms,
// for collide<.., DEV = true>); the Zou-He inlet is applied to f = h + w and shifted back.
// For float32 storage RAW changes nothing.
template <int S, bool PULL, bool RAW = false>
__device__ __forceinline__ void gather(const typename Pop<S>::T* __restrict__ f, const Grid& g,
                                       const Coef& c, int x, int y, int z, float (&v)[19]) {
    using P = Pop<S>;
    constexpr bool kRaw = RAW && P::kShifted;
    if (!PULL) {
        const long long cell = ((long long)z * g.ny + y) * g.pitch + x;
#pragma unroll
        for (int q = 0; q < 19; ++q)
            v[q] = kRaw ? P::ld_raw(f + q * g.plane + cell) : P::ld(f + q * g.plane + cell, q);
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
            const typename P::T* p = f + q * g.plane + ((long long)sz * g.ny + sy) * g.pitch + sx;
            v[q] = kRaw ? P::ld_raw(p) : P::ld(p, q);
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
template <int S>
__device__ __forceinline__ void store_raw(typename Pop<S>::T* __restrict__ f, const Grid& g,
                                          long long cell, const float (&v)[19]) {
#pragma unroll
    for (int q = 0; q < 19; ++q) Pop<S>::st_raw(f + q * g.plane + cell, v[q]);
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

// Cascaded collision in central-moment space followed by the raw-moment back transform,
// in place on f. (Fx, Fy, Fz) is the body-force density at the cell.
// DEV: f holds deviations h = f - w (shifted storage) on input and output. Moments of the
// weights are added to the zeroth and second moments (sum w = 1, sum w e_a e_b = d_ab / 3)
// and subtracted again from the raw post-collision moments before the back transform
// (sum w = 1, sum w e_a^2 = 1/3, sum w e_a^2 e_b^2 = 1/9; all other moments of w vanish),
// so no per-population shift is needed.
template <bool FORCE, bool DEV = false>
__device__ __forceinline__ void collide(float (&f)[19], const Coef& c, float Fx, float Fy,
                                        float Fz) {
    Moments m = moments(f);
    const float drho = m.rho;
    if (DEV) {
        m.rho += 1.0f;
        m.pxx += 1.0f / 3.0f;
        m.pyy += 1.0f / 3.0f;
        m.pzz += 1.0f / 3.0f;
    }
    const float r = m.rho;
    const float inv = __frcp_rn(r);
    float u = m.mx * inv, v = m.my * inv, w = m.mz * inv;
    if (FORCE) {
        u += 0.5f * Fx * inv;
        v += 0.5f * Fy * inv;
        w += 0.5f * Fz * inv;
    }
    // second-order central moments about the shifted velocity
    const float k200 = m.pxx - 2.0f * u * m.mx + u * u * r;
    const float k020 = m.pyy - 2.0f * v * m.my + v * v * r;
    const float k002 = m.pzz - 2.0f * w * m.mz + w * w * r;
    const float k110 = m.pxy - u * m.my - v * m.mx + u * v * r;
    const float k101 = m.pxz - u * m.mz - w * m.mx + u * w * r;
    const float k011 = m.pyz - v * m.mz - w * m.my + v * w * r;
    // relaxation (clbm_moving.py:170-196)
    const float k110s = k110 * c.one_m_sv, k101s = k101 * c.one_m_sv, k011s = k011 * c.one_m_sv;
    const float kA = k200 + k020 + k002;
    const float kAs = kA - c.s_e * (kA - r);
    const float kDs = (k200 - k020) * c.one_m_sv, kEs = (k200 - k002) * c.one_m_sv;
    const float k200s = (kAs + kDs + kEs) * (1.0f / 3.0f);
    const float k020s = (kAs - 2.0f * kDs + kEs) * (1.0f / 3.0f);
    const float k002s = (kAs + kDs - 2.0f * kEs) * (1.0f / 3.0f);
    // fourth-order equilibrium r/9; its weight part 1/9 is removed here in the shifted form
    const float r9 = (DEV ? drho : r) * (1.0f / 9.0f);
    // raw post-collision moments (third-order central moments relax to 0, fourth to r/9)
    const float ur = u * r, vr = v * r, wr = w * r;
    const float uu = u * u, vv = v * v, ww = w * w;
    const float T110 = k110s + u * vr, T101 = k101s + u * wr, T011 = k011s + v * wr;
    float T200 = k200s + u * ur, T020 = k020s + v * vr, T002 = k002s + w * wr;
    const float T210 = 2.0f * u * k110s + v * k200s + uu * vr;
    const float T120 = 2.0f * v * k110s + u * k020s + vv * ur;
    const float T201 = 2.0f * u * k101s + w * k200s + uu * wr;
    const float T021 = 2.0f * v * k011s + w * k020s + vv * wr;
    const float T102 = 2.0f * w * k101s + u * k002s + ww * ur;
    const float T012 = 2.0f * w * k011s + v * k002s + ww * vr;
    const float T220 = r9 + 4.0f * u * v * k110s + vv * k200s + uu * k020s + uu * vv * r;
    const float T202 = r9 + 4.0f * u * w * k101s + ww * k200s + uu * k002s + uu * ww * r;
    const float T022 = r9 + 4.0f * v * w * k011s + ww * k020s + vv * k002s + vv * ww * r;
    if (DEV) {
        T200 -= 1.0f / 3.0f; T020 -= 1.0f / 3.0f; T002 -= 1.0f / 3.0f;
    }
    // closed form of M_raw^-1 (config_moving.py:62-73)
    f[0] = (DEV ? drho : r) - (T200 + T020 + T002) + (T220 + T202 + T022);
    const float A1 = 0.5f * (T200 - T220 - T202), B1 = 0.5f * (ur - T120 - T102);
    const float A2 = 0.5f * (T020 - T220 - T022), B2 = 0.5f * (vr - T210 - T012);
    const float A3 = 0.5f * (T002 - T202 - T022), B3 = 0.5f * (wr - T201 - T021);
    f[1] = A1 + B1; f[2] = A1 - B1;
    f[3] = A2 + B2; f[4] = A2 - B2;
    f[5] = A3 + B3; f[6] = A3 - B3;
    // plane diagonals: f = (T_aabb + e_a e_b T_ab + e_b T_aab + e_a T_abb) / 4
    {
        const float s = 0.25f * T220, p = 0.25f * T110, a = 0.25f * T210, b = 0.25f * T120;
        f[7] = s + p + a + b;   // (+1,+1)
        f[8] = s - p + a - b;   // (-1,+1)
        f[9] = s - p - a + b;   // (+1,-1)
        f[10] = s + p - a - b;  // (-1,-1)
    }
    {
        const float s = 0.25f * T202, p = 0.25f * T101, a = 0.25f * T201, b = 0.25f * T102;
        f[11] = s + p + a + b;
        f[12] = s - p + a - b;
        f[13] = s - p - a + b;
        f[14] = s + p - a - b;
    }
    {
        const float s = 0.25f * T022, p = 0.25f * T011, a = 0.25f * T021, b = 0.25f * T012;
        f[15] = s + p + a + b;
        f[16] = s - p + a - b;
        f[17] = s - p - a + b;
        f[18] = s + p - a - b;
    }
    if (FORCE) {
        // Guo forcing: w_q (1 - s_v/2) [ (e - u)/cs2 + (e.u) e / cs2^2 ] . F
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const float eu = ex(q) * u + ey(q) * v + ez(q) * w;
            const float cx = (ex(q) - u) * 3.0f + eu * ex(q) * 9.0f;
            const float cy = (ey(q) - v) * 3.0f + eu * ey(q) * 9.0f;
            const float cz = (ez(q) - w) * 3.0f + eu * ez(q) * 9.0f;
            f[q] += c.wc[q] * (cx * Fx + cy * Fy + cz * Fz);
        }
    }
}

// One cell of the full-grid pass: gather, force (per FMODE), collide, store.
template <int S, bool PULL, int FMODE>
__device__ __forceinline__ void stream_collide_cell(const typename Pop<S>::T* __restrict__ fin,
                                                    typename Pop<S>::T* __restrict__ fout,
                                                    const Grid& g, const Coef& c,
                                                    const ForceArgs& fa, int x, int y, int z) {
    if (FMODE == kForceSkipBand) {
        // bulk pass of an IBM step: the cells of the force box are done by the box pass
        const Band b = band_from_box(fa.dev->box[fa.dev->cur & 1], g.nx, g.ny, g.nz);
        if (in_band(b, x, y, z, g.ny, g.nz)) return;
    }
    // shifted storage: the collision works on the deviations (no per-population shift)
    constexpr bool DEV = Pop<S>::kShifted;
    float f[19];
    gather<S, PULL, true>(fin, g, c, x, y, z, f);
    const long long cell = ((long long)z * g.ny + y) * g.pitch + x;
    if (FMODE == kForceNone || FMODE == kForceSkipBand) {
        collide<false, DEV>(f, c, 0.f, 0.f, 0.f);
    } else if (FMODE == kForceDense) {
        const float Fz = fa.fz ? fa.fz[cell] : 0.0f;
        collide<true, DEV>(f, c, fa.fx[cell], fa.fy[cell], Fz);
    } else {
        const Band b = band_from_box(fa.dev->box[fa.dev->cur & 1], g.nx, g.ny, g.nz);
        if (in_band(b, x, y, z, g.ny, g.nz)) {
            // Eulerian clip of _clip_forces (airfoil_moving.py:219-225) applied on read;
            // fz is always zero there.
            const float Fx = fminf(fmaxf(qforce(fa.qx[cell]), -0.05f), 0.05f);
            const float Fy = fminf(fmaxf(qforce(fa.qy[cell]), -0.05f), 0.05f);
            collide<true, DEV>(f, c, Fx, Fy, 0.0f);
        } else {
            collide<false, DEV>(f, c, 0.f, 0.f, 0.f);
        }
    }
    store_raw<S>(fout, g, cell, f);
}

// Forced stream-collide of the cells of the IBM force box; block bx of nbx (256 threads)
// takes cells bx * 256 + threadIdx.x, stepping by nbx * 256.
template <int S, bool PULL>
__device__ __forceinline__ void box_pass_body(const typename Pop<S>::T* __restrict__ fin,
                                              typename Pop<S>::T* __restrict__ fout,
                                              const Grid& g, const Coef& c, const ForceArgs& fa,
                                              int bx, int nbx) {
    const Band b = band_from_box(fa.dev->box[fa.dev->cur & 1], g.nx, g.ny, g.nz);
    const int cells = b.ilen * b.jlen * b.klen;
    for (int t = bx * blockDim.x + threadIdx.x; t < cells; t += nbx * blockDim.x) {
        int x, y, z;
        box_cell(b, g.ny, g.nz, t, x, y, z);
        float f[19];
        gather<S, PULL, true>(fin, g, c, x, y, z, f);
        const long long cell = ((long long)z * g.ny + y) * g.pitch + x;
        const float Fx = fminf(fmaxf(qforce(fa.qx[cell]), -0.05f), 0.05f);
        const float Fy = fminf(fmaxf(qforce(fa.qy[cell]), -0.05f), 0.05f);
        collide<true, Pop<S>::kShifted>(f, c, Fx, Fy, 0.0f);
        store_raw<S>(fout, g, cell, f);
    }
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
    const Band nb = band_from_box(dev->box[s & 1], g.nx, g.ny, g.nz);
    const Band ob = band_from_box(dev->box[(s - 1) & 1], g.nx, g.ny, g.nz);
    const int stride = nbx * blockDim.x;
    const int ocells = ob.ilen * ob.jlen * ob.klen;
    for (int t = bx * blockDim.x + threadIdx.x; t < ocells; t += stride) {
        int x, y, z;
        box_cell(ob, g.ny, g.nz, t, x, y, z);
        const long long cell = ((long long)z * g.ny + y) * g.pitch + x;
        fx[cell] = 0;
        fy[cell] = 0;
    }
    if (!compute_macro) return;
    const int ncells = nb.ilen * nb.jlen * nb.klen;
    for (int t = bx * blockDim.x + threadIdx.x; t < ncells; t += stride) {
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
        rho[cell] = r;
        ux[cell] = mx / r;
        uy[cell] = my / r;
        uz[cell] = mz / r;
    }
}

}  // namespace clbm
