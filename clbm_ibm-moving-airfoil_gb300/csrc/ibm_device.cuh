// ibm_device.cuh -- block-level bodies of the IBM kernels, shared by the single-lattice
// kernels (ibm_kernels.cu) and the batched ensemble kernels (ensemble.cu). Each body takes
// the index of its block within the lattice's launch (`bx`) and the number of such blocks
// (`nbx`) instead of blockIdx.x / gridDim.x.
#pragma once

#include "clbm_internal.cuh"

namespace clbm {


// Marker kinematics (airfoil_moving.py:100-127) of markers [bx * B, bx * B + B), B threads
// per block, and the box that bounds their 4x4x4 Peskin stencils (block min, one
// atomicMin per entry).
template <bool DEVM, int B = kMarkerBlock>
__device__ __forceinline__ void ibm_markers_body(const IbmArrays& a, const Grid& g,
                                                 const MotionF& mf, const clbm_motion& m, int bx) {
    __shared__ int sbox[B / 32][6];
    __shared__ float smot[8];
    const long long s = a.dev->step + 1;
    if (threadIdx.x == 0) {
        if (bx == 0) a.dev->cur = s;
        MotionF v = mf;
        if (DEVM) {
            // _motion_state(step), main_moving.py:65-74, in double, then the float32
            // truncation of the kernel arguments (airfoil_moving.py:101-103). One thread per
            // block: double-precision sin/cos are slow on this part.
            const double t = (double)s, w = m.w;
            v.xc = (float)m.x0;
            v.yc = (float)(m.y0 + m.a_heave * sin(w * t));
            v.theta = (float)(m.aoa0 + m.a_pitch * sin(w * t + m.phi_pitch));
            v.vx = 0.0f;
            v.vy = (float)(m.a_heave * w * cos(w * t));
            v.omega = (float)(m.a_pitch * w * cos(w * t + m.phi_pitch));
        }
        smot[0] = v.xc; smot[1] = v.yc; smot[2] = v.theta;
        smot[3] = v.vx; smot[4] = v.vy; smot[5] = v.omega;
        smot[6] = cosf(v.theta);
        smot[7] = sinf(v.theta);
    }
    __syncthreads();
    const float xc = smot[0], yc = smot[1], vx = smot[3], vy = smot[4], omega = smot[5];
    const float cos_t = smot[6], sin_t = smot[7];
    int b[6] = {kBoxEmpty, kBoxEmpty, kBoxEmpty, kBoxEmpty, kBoxEmpty, kBoxEmpty};
    const int i = bx * B + threadIdx.x;
    if (i < a.n) {
        const float x0m = a.X0[i], y0m = a.Y0[i], zk = a.Z0[i];
        const float xk = xc + x0m * cos_t - y0m * sin_t;
        const float yk = yc + x0m * sin_t + y0m * cos_t;
        a.X[i] = xk;
        a.Y[i] = yk;
        a.Z[i] = zk;
        const float rx = xk - xc, ry = yk - yc;
        a.VX[i] = vx - omega * ry;
        a.VY[i] = vy + omega * rx;
        const int ib = (int)floorf(xk) - 1, jb = (int)floorf(yk) - 1, kb = (int)floorf(zk) - 1;
        b[0] = min(max(ib, 0), g.nx - 1);
        b[1] = -min(max(ib + 3, 0), g.nx - 1);
        b[2] = jb;
        b[3] = -(jb + 3);
        b[4] = kb;
        b[5] = -(kb + 3);
    }
#pragma unroll
    for (int e = 0; e < 6; ++e) b[e] = __reduce_min_sync(0xffffffffu, b[e]);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int e = 0; e < 6; ++e) sbox[warp][e] = b[e];
    __syncthreads();
    if (threadIdx.x < 6) {
        int v = sbox[0][threadIdx.x];
        for (int w = 1; w < B / 32; ++w) v = min(v, sbox[w][threadIdx.x]);
        if (v != kBoxEmpty) atomicMin(&a.dev->box[s & 1][threadIdx.x], v);
        __threadfence();
    }
    // the last of the launch's ceil(n / 256) blocks converts the finished box to its band
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int nbx = (unsigned int)((a.n + B - 1) / B);
        last = atomicAdd(&a.dev->mticket, 1u) == nbx - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        int bx6[6];
        for (int e = 0; e < 6; ++e) bx6[e] = atomicAdd(&a.dev->box[s & 1][e], 0);
        const Band b = band_from_box(bx6, g.nx, g.ny, g.nz);
        int* o = a.dev->band[s & 1];
        o[0] = b.i0; o[1] = b.ilen; o[2] = b.j0; o[3] = b.jlen; o[4] = b.k0; o[5] = b.klen;
        a.dev->mticket = 0u;
    }
}

// Stencil taps of one marker held by a lane (two of the 64), with the marker's force.
struct MarkerTaps {
    float wt[2];      // Peskin weight of tap h
    int ii[2];        // x index (clamped)
    int jr[2], kr[2]; // y, z index before the periodic wrap
    float fx, fy;     // clipped marker force
};

// Fire-and-forget 64-bit add to a global force field (a reduction: no value comes back).
__device__ __forceinline__ void red_add(long long* p, long long v) {
    asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Spreading contribution of tap h in 64-bit fixed point: the float32 product f * w
// (airfoil_moving.py:212-214) scaled by 2^40, so sums do not depend on their order.
__device__ __forceinline__ long long spread_q(float f, float w) {
    return __float2ll_rn(f * w * kForceScale);
}

// Markers m0 .. m0 + K - 1 (those below a.n: has[k], warp-uniform) on one warp: Peskin
// interpolation of the current velocity (two stencil taps per lane, warp-shuffle sums;
// airfoil_moving.py:142-170) and the marker force clip (airfoil_moving.py:175-183). The
// velocity gathers of all K markers are issued before any of their sums, so a warp has K
// times the loads in flight; the taps are kept for spreading.
// PERM: entries m0 .. m0 + K - 1 of the marker order a.perm instead of the markers
// themselves (every output goes to the marker's own index, so the results do not depend
// on the order).
template <int K, bool PERM = false>
__device__ __forceinline__ void ibm_interp_markers(const IbmArrays& a, const Grid& g, int m0, int lane,
                                                   MarkerTaps (&tp)[K], bool (&has)[K]) {
    float xk[K], yk[K], zk[K], vxk[K], vyk[K], us[K], vs[K], uxv[K][2], uyv[K][2];
    int mk[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        has[k] = m0 + k < a.n;
        const int j = has[k] ? m0 + k : 0;   // launched only with a.n >= 1
        const int m = PERM ? a.perm[j] : j;
        mk[k] = m;
        xk[k] = a.X[m]; yk[k] = a.Y[m]; zk[k] = a.Z[m];
        vxk[k] = a.VX[m]; vyk[k] = a.VY[m];   // with the positions: one round trip less
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int ib = (int)floorf(xk[k]) - 1, jb = (int)floorf(yk[k]) - 1, kb = (int)floorf(zk[k]) - 1;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            // tap t: di fastest, so four neighbouring lanes read four consecutive x
            const int t = lane + 32 * h;
            const int di = t & 3, dj = (t >> 2) & 3, dk = t >> 4;
            const int ii = min(max(ib + di, 0), g.nx - 1);   // x clamped (airfoil_moving.py:158)
            const int jj = pmod(jb + dj, g.ny);              // y, z periodic indices; the weight
            const int kk = pmod(kb + dk, g.nz);              // uses the wrapped index, as there
            const float w = phi1d((float)ii - xk[k]) * phi1d((float)jj - yk[k]) * phi1d((float)kk - zk[k]);
            const long long c = ((long long)kk * g.ny + jj) * g.pitch + ii;
            tp[k].wt[h] = w;
            tp[k].ii[h] = ii;
            tp[k].jr[h] = jb + dj;
            tp[k].kr[h] = kb + dk;
            const bool ok = w != 0.0f && in_bounds(c, g.plane, g.status);
            uxv[k][h] = ok ? a.ux[c] : 0.0f;
            uyv[k][h] = ok ? a.uy[c] : 0.0f;
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        us[k] = 0.f;
        vs[k] = 0.f;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (tp[k].wt[h] != 0.0f) {
                us[k] += uxv[k][h] * tp[k].wt[h];
                vs[k] += uyv[k][h] * tp[k].wt[h];
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            us[k] += __shfl_xor_sync(0xffffffffu, us[k], o);
            vs[k] += __shfl_xor_sync(0xffffffffu, vs[k], o);
        }
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (!has[k]) continue;
        const int m = mk[k];
        tp[k].fx = fmaxf(-0.05f, fminf(0.05f, -(us[k] - vxk[k])));
        tp[k].fy = fmaxf(-0.05f, fminf(0.05f, -(vs[k] - vyk[k])));
        if (lane == 0) {
            a.Uk[m] = us[k];
            a.Vk[m] = vs[k];
            a.FXk[m] = tp[k].fx;
            a.FYk[m] = tp[k].fy;
        }
    }
}

// K markers per warp: interpolation, then spreading with one global reduction per tap and
// component.
template <int K>
__device__ __forceinline__ void ibm_interp_spread_body(const IbmArrays& a, const Grid& g, int m0,
                                                       int lane) {
    MarkerTaps tp[K];
    bool has[K];
    ibm_interp_markers<K>(a, g, m0, lane, tp, has);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if (!has[k]) continue;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (tp[k].wt[h] != 0.0f) {
                const long long c = ((long long)pmod(tp[k].kr[h], g.nz) * g.ny + pmod(tp[k].jr[h], g.ny)) * g.pitch + tp[k].ii[h];
                if (!in_bounds(c, g.plane, g.status)) continue;
                red_add(a.fx + c, spread_q(tp[k].fx, tp[k].wt[h]));
                red_add(a.fy + c, spread_q(tp[k].fy, tp[k].wt[h]));
            }
        }
    }
}

// Spreading through a shared-memory tile: a block of 8 warps takes kTileMarkers
// consecutive entries of the marker order a.perm (markers sorted by their body-frame cell,
// so they lie close together), interpolates them (four per warp, as above), accumulates their int64
// contributions in a tile over the box their stencils cover (y, z before the wrap) and
// adds each touched cell to the global fields once. The sums are the same integers as with
// one global atomic per tap. A chunk whose box exceeds the tile (or spans the lattice in
// y or z) spreads with direct global atomics.
constexpr int kTileMarkers = 32;
constexpr int kTileCells = 2048;   // two int64 per cell: 32 KB of shared memory
constexpr int kTileMarkersPerWarp = kTileMarkers / (kTiledBlock / 32);

__device__ __forceinline__ void ibm_interp_spread_tiled_body(const IbmArrays& a, const Grid& g, int chunk) {
    __shared__ long long tfx[kTileCells], tfy[kTileCells];
    __shared__ int sb[6];   // box, inclusive: imin, -imax, jmin, -jmax, kmin, -kmax
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x < 6) sb[threadIdx.x] = 0x7fffffff;
    __syncthreads();
    MarkerTaps tp[kTileMarkersPerWarp];
    bool has[kTileMarkersPerWarp];
    ibm_interp_markers<kTileMarkersPerWarp, true>(a, g, chunk * kTileMarkers + warp * kTileMarkersPerWarp,
                                                  lane, tp, has);
#pragma unroll
    for (int i = 0; i < kTileMarkersPerWarp; ++i) {
        if (has[i]) {
            // taps 0 and 63 hold the stencil's corners (di, dj, dk = 0 and 3)
            if (lane == 0) {
                atomicMin(&sb[0], tp[i].ii[0]);
                atomicMin(&sb[2], tp[i].jr[0]);
                atomicMin(&sb[4], tp[i].kr[0]);
            } else if (lane == 31) {
                atomicMin(&sb[1], -tp[i].ii[1]);
                atomicMin(&sb[3], -tp[i].jr[1]);
                atomicMin(&sb[5], -tp[i].kr[1]);
            }
        }
    }
    __syncthreads();
    const int i0 = sb[0], j0 = sb[2], k0 = sb[4];
    const int li = -sb[1] - i0 + 1, lj = -sb[3] - j0 + 1, lk = -sb[5] - k0 + 1;
    const bool tiled = sb[0] != 0x7fffffff && lj < g.ny && lk < g.nz &&
                       (long long)li * lj * lk <= kTileCells;   // block-uniform
    if (!tiled) {
#pragma unroll
        for (int i = 0; i < kTileMarkersPerWarp; ++i) {
            if (!has[i]) continue;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (tp[i].wt[h] != 0.0f) {
                    const long long c = ((long long)pmod(tp[i].kr[h], g.nz) * g.ny + pmod(tp[i].jr[h], g.ny)) * g.pitch + tp[i].ii[h];
                    if (!in_bounds(c, g.plane, g.status)) continue;
                    red_add(a.fx + c, spread_q(tp[i].fx, tp[i].wt[h]));
                    red_add(a.fy + c, spread_q(tp[i].fy, tp[i].wt[h]));
                }
            }
        }
        return;
    }
    const int vol = li * lj * lk;
    for (int t = threadIdx.x; t < vol; t += kTiledBlock) {
        tfx[t] = 0;
        tfy[t] = 0;
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kTileMarkersPerWarp; ++i) {
        if (!has[i]) continue;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (tp[i].wt[h] != 0.0f) {
                const int l = (tp[i].ii[h] - i0) + li * ((tp[i].jr[h] - j0) + lj * (tp[i].kr[h] - k0));
                atomicAdd(reinterpret_cast<unsigned long long*>(tfx + l), (unsigned long long)spread_q(tp[i].fx, tp[i].wt[h]));
                atomicAdd(reinterpret_cast<unsigned long long*>(tfy + l), (unsigned long long)spread_q(tp[i].fy, tp[i].wt[h]));
            }
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < vol; t += kTiledBlock) {
        const long long vx = tfx[t], vy = tfy[t];
        if (vx == 0 && vy == 0) continue;
        const int x = i0 + t % li;
        const int r = t / li;
        const int y = pmod(j0 + r % lj, g.ny), z = pmod(k0 + r / lj, g.nz);
        const long long c = ((long long)z * g.ny + y) * g.pitch + x;
        if (!in_bounds(c, g.plane, g.status)) continue;
        if (vx) red_add(a.fx + c, vx);
        if (vy) red_add(a.fy + c, vy);
    }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Double sums of the clipped Eulerian force over the box and of the marker forces into the
// history ring, then the device call counter advances. Block bx of nbx writes its partial;
// the last block to finish sums the partials in block order (scheduling-independent).
template <int B = kFinishBlock>
__device__ __forceinline__ void ibm_finish_body(const IbmArrays& a, const Grid& g, int bx, int nbx) {
    __shared__ double red[B / 32][4];
    __shared__ bool last;
    IbmDev* dev = a.dev;
    const long long s = dev->step + 1;
    const Band b = load_band(dev, (int)(s & 1));
    const int cells = b.ilen * b.jlen * b.klen;
    const int stride = nbx * B;
    // Every clipped Eulerian value is an integer multiple of 2^-40 (a float of the int64
    // field times 2^-40, or the float 0.05f = 13421773 * 2^-28) of magnitude <= 0.05. The
    // integers k = value * 2^40 are summed exactly in int64 and converted once: the exact
    // sum rounded to double, which is also what adding the values in double gives, in any
    // order, while the partial sums stay below 2^13 (every add is then exact); this keeps
    // the slow double-precision adds of this part to one per block.
    long long kx = 0, ky = 0;
    double mx = 0.0, my = 0.0;
    for (int t = bx * B + threadIdx.x; t < cells; t += stride) {
        int x, y, z;
        box_cell(b, g.ny, g.nz, t, x, y, z);
        const long long c = ((long long)z * g.ny + y) * g.pitch + x;
        kx += (long long)(fminf(fmaxf(qforce(a.fx[c]), -0.05f), 0.05f) * kForceScale);
        ky += (long long)(fminf(fmaxf(qforce(a.fy[c]), -0.05f), 0.05f) * kForceScale);
    }
    for (int t = bx * B + threadIdx.x; t < a.n; t += stride) {
        mx += (double)a.FXk[t];
        my += (double)a.FYk[t];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        kx += __shfl_xor_sync(0xffffffffu, kx, o);
        ky += __shfl_xor_sync(0xffffffffu, ky, o);
    }
    const double sx = (double)kx * (double)kForceInvScale, sy = (double)ky * (double)kForceInvScale;
    mx = warp_sum(mx); my = warp_sum(my);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { red[warp][0] = sx; red[warp][1] = sy; red[warp][2] = mx; red[warp][3] = my; }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0.0;
        for (int w = 0; w < B / 32; ++w) v += red[w][threadIdx.x];
        a.part[4 * bx + threadIdx.x] = v;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int tk = atomicAdd(&dev->ticket, 1u);
        last = (tk == (unsigned int)nbx - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int blk = threadIdx.x; blk < nbx; blk += B)
        for (int e = 0; e < 4; ++e) v[e] += __ldcg(a.part + 4 * blk + e);
    for (int e = 0; e < 4; ++e) v[e] = warp_sum(v[e]);
    __syncthreads();
    if (lane == 0)
        for (int e = 0; e < 4; ++e) red[warp][e] = v[e];
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int w = 0; w < B / 32; ++w) t += red[w][threadIdx.x];
        a.hist[4 * ((s - 1) % a.hist_cap) + threadIdx.x] = t;
    }
    if (threadIdx.x == 0) {
        dev->ticket = 0u;
        // the previous call's box was consumed by this call's band-prepare
        for (int e = 0; e < 6; ++e) dev->box[(s + 1) & 1][e] = kBoxEmpty;
        __threadfence();
        dev->step = s;
    }
}

// Force sums folded into the box pass (single lattice): each block of the box pass brings
// the integer sums kx, ky of its cells' clipped Eulerian force (units of 2^-40); they are
// added exactly into dev->ksum. The marker forces are summed in double by the first
// P = min(blocks, kFinishBlocks) blocks, block b over its own contiguous share of the
// markers (thread-strided, warp butterfly, warps in order), into a.part; the last block to
// finish adds the P partials in block order, converts the integer sums, writes the history
// entry of the call whose box this was and advances the device call counter -- the work of
// ibm_finish_body without its own launch. The Eulerian part is the same exact integer sum;
// the marker part is the same set of doubles added in another fixed order. (One block
// summing all markers would wait on one load round trip per marker and thread: 197 of them
// at 12,600 markers and 64 threads.)
__device__ __forceinline__ void ibm_box_sums_tail(const IbmArrays& a, long long kx, long long ky) {
    __shared__ long long kred[32][2];
    __shared__ double dred[32][2];
    __shared__ bool last;
    IbmDev* dev = a.dev;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int P = min((int)gridDim.x, kFinishBlocks);
    if ((int)blockIdx.x < P) {
        const int chunk = (a.n + P - 1) / P;
        const int m0 = (int)blockIdx.x * chunk, m1 = min(a.n, m0 + chunk);
        double mx = 0.0, my = 0.0;
#pragma unroll 4
        for (int m = m0 + (int)threadIdx.x; m < m1; m += blockDim.x) {
            mx += (double)a.FXk[m];
            my += (double)a.FYk[m];
        }
        mx = warp_sum(mx);
        my = warp_sum(my);
        if (lane == 0) { dred[warp][0] = mx; dred[warp][1] = my; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        kx += __shfl_xor_sync(0xffffffffu, kx, o);
        ky += __shfl_xor_sync(0xffffffffu, ky, o);
    }
    if (lane == 0) { kred[warp][0] = kx; kred[warp][1] = ky; }
    __syncthreads();
    if (threadIdx.x == 0) {
        if ((int)blockIdx.x < P) {
            double tx = 0.0, ty = 0.0;
            for (int w = 0; w < nw; ++w) { tx += dred[w][0]; ty += dred[w][1]; }
            a.part[2 * blockIdx.x] = tx;
            a.part[2 * blockIdx.x + 1] = ty;
        }
        long long sx = 0, sy = 0;
        for (int w = 0; w < nw; ++w) { sx += kred[w][0]; sy += kred[w][1]; }
        if (sx) atomicAdd((unsigned long long*)&dev->ksum[0], (unsigned long long)sx);
        if (sy) atomicAdd((unsigned long long*)&dev->ksum[1], (unsigned long long)sy);
        __threadfence();
        last = atomicAdd(&dev->bticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double mx = 0.0, my = 0.0;
    for (int b = threadIdx.x; b < P; b += blockDim.x) {
        mx += __ldcg(a.part + 2 * b);
        my += __ldcg(a.part + 2 * b + 1);
    }
    mx = warp_sum(mx);
    my = warp_sum(my);
    __syncthreads();   // dred is reused
    if (lane == 0) { dred[warp][0] = mx; dred[warp][1] = my; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double tx = 0.0, ty = 0.0;
        for (int w = 0; w < nw; ++w) { tx += dred[w][0]; ty += dred[w][1]; }
        const long long s = dev->step + 1;
        const long long ex = (long long)__ldcg((const unsigned long long*)&dev->ksum[0]);
        const long long ey = (long long)__ldcg((const unsigned long long*)&dev->ksum[1]);
        double* h = a.hist + 4 * ((s - 1) % a.hist_cap);
        h[0] = (double)ex * (double)kForceInvScale;
        h[1] = (double)ey * (double)kForceInvScale;
        h[2] = tx;
        h[3] = ty;
        dev->ksum[0] = 0;
        dev->ksum[1] = 0;
        dev->bticket = 0u;
        // the previous call's box was consumed by this call's band-prepare
        for (int e = 0; e < 6; ++e) dev->box[(s + 1) & 1][e] = kBoxEmpty;
        __threadfence();
        dev->step = s;
    }
}

}  // namespace clbm
