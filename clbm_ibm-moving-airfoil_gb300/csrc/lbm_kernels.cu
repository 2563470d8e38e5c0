// lbm_kernels.cu -- fused pull-stream + cascaded central-moment collision for D3Q19.
//
// One pass per time step. Each thread owns one cell (x fastest, so a warp covers 32
// consecutive x of one row) and
//   1. pulls its 19 post-stream populations from the post-collision state of the
//      previous step, f(x) = f_post(x - e_q) with y/z periodic wrap (clbm_moving.py:254-261),
//      the zero-gradient outlet folded in as "cell Nx-1 pulls like cell Nx-2"
//      (clbm_moving.py:296-300) and the Zou-He velocity inlet applied in registers at
//      x = 0 (clbm_moving.py:266-294);
//   2. takes rho and the half-force-shifted velocity (clbm_moving.py:96-115);
//   3. relaxes the second-order central moments and rebuilds the raw moments with the
//      reference's fixed choices s_q = s_pi = 1 (clbm_moving.py:170-231);
//   4. maps raw moments back to populations with the closed form of M_raw^-1 (entries
//      0, +-1/4, +-1/2, +-1; clbm_moving.py:233-238) and adds Guo forcing
//      (clbm_moving.py:240-249) where the force is non-zero;
//   5. stores f_post for the next step, coalesced (plain stores: the streaming hint measured slower).
// Algorithmic traffic: 19 loads + 19 stores per cell (152 B/cell float32, 76 B/cell for
// the 16-bit shifted forms); the force fields add 8 B per cell inside the IBM band only.
#include <algorithm>
#include <cstdlib>

#include "ibm_device.cuh"
#include "lbm_device.cuh"

namespace clbm {

constexpr int kBX = 128;  // threads per block along x

template <int S, bool PULL, int FMODE, bool IDX32>
__global__ void __launch_bounds__(kBX) k_stream_collide(const typename Pop<S>::T* __restrict__ fin,
                                                        typename Pop<S>::T* __restrict__ fout,
                                                        Grid g, Coef c, ForceArgs fa) {
    const int x = blockIdx.x * kBX + threadIdx.x;
    if (x >= g.nx) return;
    stream_collide_cell<S, PULL, FMODE, IDX32>(fin, fout, g, c, fa, x, blockIdx.y, blockIdx.z);
}

// Forced pass over the cells of the IBM force box (the complement of the bulk pass), by
// rows of the box. Work item w is x segment w % nseg of row w / nseg of the box's (y, z)
// rows, nseg from the box's x extent; the blocks step through the items (grid-stride,
// grid sized by the host from the box bound), so no block is launched for rows the box
// does not have. Along a row the cells are consecutive, so the pass uses the bulk pass's
// coalesced bodies: two cells per thread from x = i0 rounded down to even in the 16-bit
// forms (pair_body), one cell per thread from i0 in float32 (stream_collide_cell); cells
// outside the box are left to the bulk pass. SUMS: the block's integer force sums go to
// ibm_box_sums_tail (force sums of the call whose box this is, history ring, call
// counter).
template <int S, bool PULL, bool SUMS, bool IDX32>
__global__ void __launch_bounds__(kBoxBlock, 16) k_box_rows_pair(const typename Pair<S>::T* __restrict__ fin,
                                                                 typename Pair<S>::T* __restrict__ fout,
                                                                 Grid g, Coef c, ForceArgs fa, IbmArrays a) {
    const Band b = load_band(fa.dev, fa.slot);
    const int xa = b.i0 & ~1;
    const int nseg = (b.i0 + b.ilen - xa + 2 * kBoxBlock - 1) / (2 * kBoxBlock);
    const int items = nseg * b.jlen * b.klen;
    long long ks[2] = {0, 0};
    for (int w = blockIdx.x; w < items; w += gridDim.x) {   // block-uniform
        const int seg = w % nseg, r = w / nseg;
        const int y = pmod(b.j0 + r % b.jlen, g.ny), z = pmod(b.k0 + r / b.jlen, g.nz);
        pair_body<S, PULL, kForceOnlyBand, IDX32>(fin, fout, g, c, fa,
                                                  xa + seg * 2 * kBoxBlock + 2 * (int)threadIdx.x, y, z,
                                                  SUMS ? ks : nullptr);
    }
    if (SUMS) ibm_box_sums_tail(a, ks[0], ks[1]);
}

template <int S, bool PULL, bool SUMS>
__global__ void __launch_bounds__(kBoxBlock, 8) k_box_rows_cell(const typename Pop<S>::T* __restrict__ fin,
                                                                typename Pop<S>::T* __restrict__ fout,
                                                                Grid g, Coef c, ForceArgs fa, IbmArrays a) {
    const Band b = load_band(fa.dev, fa.slot);
    const int nseg = (b.ilen + kBoxBlock - 1) / kBoxBlock;
    const int items = nseg * b.jlen * b.klen;
    long long ks[2] = {0, 0};
    for (int w = blockIdx.x; w < items; w += gridDim.x) {
        const int seg = w % nseg, r = w / nseg;
        const int x = b.i0 + seg * kBoxBlock + (int)threadIdx.x;
        const int y = pmod(b.j0 + r % b.jlen, g.ny), z = pmod(b.k0 + r / b.jlen, g.nz);
        if (x < b.i0 + b.ilen)
            stream_collide_cell<S, PULL, kForceOnlyBand>(fin, fout, g, c, fa, x, y, z, SUMS ? ks : nullptr);
    }
    if (SUMS) ibm_box_sums_tail(a, ks[0], ks[1]);
}

// ------------------------------------------------------------------ 16-bit pair kernel
// Two cells per thread (Pair, pair_body in lbm_device.cuh).
// PX threads per block (2 PX cells along x): 32, 64 or 128, whichever leaves fewer idle
// lanes at the row ends (pair_threads; 64 on a tie with 32).
template <int S, bool PULL, int FMODE, int PX, bool IDX32>
__global__ void __launch_bounds__(PX, 1024 / PX) k_stream_collide_pair(const typename Pair<S>::T* __restrict__ fin,
                                                                    typename Pair<S>::T* __restrict__ fout,
                                                                    Grid g, Coef c, ForceArgs fa) {
    pair_body<S, PULL, FMODE, IDX32>(fin, fout, g, c, fa, 2 * (blockIdx.x * PX + threadIdx.x), blockIdx.y,
                                     blockIdx.z);
}

static int pair_threads(int nx) {
    const int w32 = (nx + 63) / 64 * 64 - nx, w64 = (nx + 127) / 128 * 128 - nx,
              w128 = (nx + 255) / 256 * 256 - nx;
    if (w32 < w64) return 32;   // narrow rows (150, 300 cells): 64 cells per block
    return w64 < w128 ? 64 : 128;
}

template <int S, bool PULL, int PX, bool IDX32>
static void pair_launch_i(int fmode, const void* fin, void* fout, const Grid& g, const Coef& c,
                          const ForceArgs& fa, cudaStream_t st) {
    using T = typename Pair<S>::T;
    const dim3 grid((g.nx + 2 * PX - 1) / (2 * PX), g.ny, g.nz);
    if (fmode == kForceNone)
        k_stream_collide_pair<S, PULL, kForceNone, PX, IDX32><<<grid, PX, 0, st>>>((const T*)fin, (T*)fout, g, c, fa);
    else if (fmode == kForceBand)
        k_stream_collide_pair<S, PULL, kForceBand, PX, IDX32><<<grid, PX, 0, st>>>((const T*)fin, (T*)fout, g, c, fa);
    else if (fmode == kForceSkipBand)
        k_stream_collide_pair<S, PULL, kForceSkipBand, PX, IDX32><<<grid, PX, 0, st>>>((const T*)fin, (T*)fout, g, c, fa);
    else
        k_stream_collide_pair<S, PULL, kForceDense, PX, IDX32><<<grid, PX, 0, st>>>((const T*)fin, (T*)fout, g, c, fa);
}

// 32-bit element indices while every index of the 19 planes fits (one wide multiply-add
// per address instead of 64-bit index arithmetic).
template <int S, bool PULL, int PX>
static void pair_launch(int fmode, const void* fin, void* fout, const Grid& g, const Coef& c,
                        const ForceArgs& fa, cudaStream_t st) {
    if (19LL * g.plane <= 0xffffffffLL) pair_launch_i<S, PULL, PX, true>(fmode, fin, fout, g, c, fa, st);
    else pair_launch_i<S, PULL, PX, false>(fmode, fin, fout, g, c, fa, st);
}

// ------------------------------------------------------------------ TMA-staged kernel
// Bulk stream-collide with the pulled rows staged in shared memory by the tensor memory
// accelerator. A block owns `seg` cells of one (y, z) row. One thread issues, for each of
// the 19 populations, a 1-D bulk copy (cp.async.bulk) of the source row of that population
// (the row at y - e_y, z - e_z) over x in [xs - 8, xs + seg + 8), completing on one
// mbarrier; every address and size is a multiple of 16 bytes (rows are padded to 32
// elements, segments and halos are multiples of 8 elements). Each thread then computes two
// neighbouring cells, reading the x-shifted populations from shared memory at constant
// offsets, and stores its results directly (coalesced), so cells of the IBM force box can
// be left to the box pass cell by cell.
template <int S> struct Stg;
template <> struct Stg<CLBM_STORE_F32> {
    using T = float;
    static constexpr bool kDev = false;
    static __device__ __forceinline__ float2 lds2(const T* p) { return *reinterpret_cast<const float2*>(p); }
    static __device__ __forceinline__ float lds1(const T* p) { return *p; }
    static __device__ __forceinline__ void st2(T* p, float a, float b) {
        *reinterpret_cast<float2*>(p) = make_float2(a, b);
    }
    static __device__ __forceinline__ void st1(T* p, float a) { *p = a; }
};
template <> struct Stg<CLBM_STORE_F16S> {
    using T = __half;
    static constexpr bool kDev = true;
    static __device__ __forceinline__ float2 lds2(const T* p) {
        return __half22float2(*reinterpret_cast<const __half2*>(p));
    }
    static __device__ __forceinline__ float lds1(const T* p) { return __half2float(*p); }
    static __device__ __forceinline__ void st2(T* p, float a, float b) { Pair<CLBM_STORE_F16S>::st2(p, a, b); }
    static __device__ __forceinline__ void st1(T* p, float a) { Pair<CLBM_STORE_F16S>::st1(p, a); }
};
template <> struct Stg<CLBM_STORE_BF16S> {
    using T = __nv_bfloat16;
    static constexpr bool kDev = true;
    static __device__ __forceinline__ float2 lds2(const T* p) {
        return __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(p));
    }
    static __device__ __forceinline__ float lds1(const T* p) { return __bfloat162float(*p); }
    static __device__ __forceinline__ void st2(T* p, float a, float b) { Pair<CLBM_STORE_BF16S>::st2(p, a, b); }
    static __device__ __forceinline__ void st1(T* p, float a) { Pair<CLBM_STORE_BF16S>::st1(p, a); }
};

constexpr int kHalo = 8;                 // elements staged on each side of a segment

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

template <int S, bool PULL, int FMODE>
__global__ void __launch_bounds__(256) k_stream_collide_tma(const typename Stg<S>::T* __restrict__ fin,
                                                            typename Stg<S>::T* __restrict__ fout,
                                                            Grid g, Coef c, ForceArgs fa) {
    using P = Stg<S>;
    using T = typename P::T;
    constexpr bool DEV = P::kDev;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long mbar;
    T* tile = reinterpret_cast<T*>(smem_raw);
    const int ld = g.seg + 2 * kHalo;               // staged elements per population
    const int xs = blockIdx.x * g.seg;
    const int y = blockIdx.y, z = blockIdx.z;
    const int t = threadIdx.x;
    const unsigned bar = smem_u32(&mbar);
    if (t == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        const int xl = max(xs - kHalo, 0);
        const int xr = min(xs + g.seg + kHalo, g.pitch);
        const unsigned bytes = (unsigned)(xr - xl) * (unsigned)sizeof(T);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                     ::"r"(bar), "r"(bytes * 19u + (unsigned)g.extra_tx) : "memory");
        const int ym = (y == 0) ? g.ny - 1 : y - 1;
        const int yp = (y == g.ny - 1) ? 0 : y + 1;
        const int zm = (z == 0) ? g.nz - 1 : z - 1;
        const int zp = (z == g.nz - 1) ? 0 : z + 1;
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            const int sy = PULL ? (ey(q) == 1 ? ym : (ey(q) == -1 ? yp : y)) : y;
            const int sz = PULL ? (ez(q) == 1 ? zm : (ez(q) == -1 ? zp : z)) : z;
            const T* src = fin + q * g.plane + ((long long)sz * g.ny + sy) * g.pitch + xl;
            const unsigned dst = smem_u32(tile + q * ld + (xl - (xs - kHalo)));
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                ::"r"(dst), "l"(src), "r"(bytes), "r"(bar) : "memory");
        }
    }
    __syncthreads();  // barrier initialised before anyone polls it
    const int x0 = xs + 2 * t;
    if (x0 >= g.nx || t * 2 >= g.seg) return;
    const bool act1 = x0 + 1 < g.nx;
    bool in0 = false, in1 = false;
    if (FMODE == kForceSkipBand || FMODE == kForceBand) {
        const Band b = load_band(fa.dev, fa.slot);
        in0 = in_band(b, x0, y, z, g.ny, g.nz);
        in1 = act1 && in_band(b, x0 + 1, y, z, g.ny, g.nz);
    }
    const bool use0 = !(FMODE == kForceSkipBand && in0);
    const bool use1 = act1 && !(FMODE == kForceSkipBand && in1);
    // bounded wait for the staged rows
    unsigned done = 0;
    for (int it = 0; it < g.spin_limit && !done; ++it) {
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
            : "=r"(done) : "r"(bar) : "memory");
    }
    if (!done) {
        atomicOr(g.status, kStatusWaitTimeout);
        return;
    }
    if (!use0 && !use1) return;
    const int i0 = kHalo + 2 * t;  // staged index of cell x0
    float h0[19], h1[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const T* r = tile + q * ld + i0;
        if (!PULL || ex(q) == 0) {
            const float2 p = P::lds2(r);
            h0[q] = p.x;
            h1[q] = p.y;
        } else if (ex(q) == 1) {
            h0[q] = P::lds1(r - 1);   // at x0 = 0 an inlet unknown, rebuilt by Zou-He below
            h1[q] = P::lds1(r);
        } else {
            h0[q] = P::lds1(r + 1);
            h1[q] = P::lds1(r + 2);
        }
    }
    if (PULL) {
        if (x0 == 0) {
            if (DEV) {
#pragma unroll
                for (int q = 0; q < 19; ++q) h0[q] += wq(q);
            }
            zou_he(h0, c);
            if (DEV) {
#pragma unroll
                for (int q = 0; q < 19; ++q) h0[q] -= wq(q);
            }
        }
        if (x0 + 1 == g.nx - 1) {
            // outlet column Nx-1 is a copy of column Nx-2 = x0 (clbm_moving.py:296-300)
#pragma unroll
            for (int q = 0; q < 19; ++q) h1[q] = h0[q];
        } else if (x0 == g.nx - 1) {
            // odd Nx: the outlet is the first cell of the last pair; pull like column Nx-2
#pragma unroll
            for (int q = 0; q < 19; ++q) h0[q] = P::lds1(tile + q * ld + i0 - 1 - ex(q));
        }
    }
    const long long row = ((long long)z * g.ny + y) * g.pitch;
    float F0x = 0.f, F0y = 0.f, F0z = 0.f, F1x = 0.f, F1y = 0.f, F1z = 0.f;
    bool frc0 = false, frc1 = false;
    if (FMODE == kForceBand) {
        frc0 = in0;
        frc1 = in1;
        if (in0) {
            F0x = fminf(fmaxf(qforce(fa.qx[row + x0]), -0.05f), 0.05f);
            F0y = fminf(fmaxf(qforce(fa.qy[row + x0]), -0.05f), 0.05f);
        }
        if (in1) {
            F1x = fminf(fmaxf(qforce(fa.qx[row + x0 + 1]), -0.05f), 0.05f);
            F1y = fminf(fmaxf(qforce(fa.qy[row + x0 + 1]), -0.05f), 0.05f);
        }
    } else if (FMODE == kForceDense) {
        frc0 = true;
        frc1 = act1;
        F0x = fa.fx[row + x0]; F0y = fa.fy[row + x0]; F0z = fa.fz ? fa.fz[row + x0] : 0.f;
        if (act1) {
            F1x = fa.fx[row + x0 + 1]; F1y = fa.fy[row + x0 + 1];
            F1z = fa.fz ? fa.fz[row + x0 + 1] : 0.f;
        }
    }
    collide_pair<DEV>(h0, h1, c, use0, use1, frc0, frc1, F0x, F0y, F0z, F1x, F1y, F1z);
    T* o = fout + row + x0;
    if (use0 && use1) {
#pragma unroll
        for (int q = 0; q < 19; ++q) P::st2(o + q * g.plane, h0[q], h1[q]);
    } else {
        if (use0) {
#pragma unroll
            for (int q = 0; q < 19; ++q) P::st1(o + q * g.plane, h0[q]);
        }
        if (use1) {
#pragma unroll
            for (int q = 0; q < 19; ++q) P::st1(o + q * g.plane + 1, h1[q]);
        }
    }
}

// Threads per block (two cells each) of the staged kernel for a lattice width: the widest
// block whose segments waste at most as many lanes as any narrower choice.
int staged_segment(int nx) {
    int best = 64, best_waste = 1 << 30;
    for (int th = 64; th <= 256; th += 32) {
        const int seg = 2 * th;
        const int nseg = (nx + seg - 1) / seg;
        const int waste = nseg * seg - nx;
        if (waste <= best_waste) {
            best_waste = waste;
            best = seg;
        }
    }
    return best;
}

template <int S>
__global__ void k_init(typename Pop<S>::T* __restrict__ f, Grid g, Coef c) {
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    // _init_feq, clbm_moving.py:75-91 (same operation order)
    const float ux0 = c.ux_in, uy0 = c.uy_in;
    const float cs2 = 1.0f / 3.0f, cs4 = (float)((1.0 / 3.0) * (1.0 / 3.0));
    const float u2 = ux0 * ux0 + uy0 * uy0;
    const long long cell = ((long long)z * g.ny + y) * g.pitch + x;
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const float eu = (float)ex(q) * ux0 + (float)ey(q) * uy0;
        const float v = wq(q) * (1.0f + eu / cs2 + 0.5f * eu * eu / cs4 - 0.5f * u2 / cs2);
        Pop<S>::st(f + q * g.plane + cell, q, v);
    }
}

__device__ __forceinline__ unsigned int ordered(float v) {
    unsigned int u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// _macro_post (clbm_moving.py:305-321) over the whole grid, plus divergence statistics.
// Grid-stride over row segments of kBX cells: a block of kBX threads takes segments
// blockIdx.x, blockIdx.x + gridDim.x, ... (segment t: x block t % nxb, row t / nxb), keeps
// its statistics in registers, and reduces them once at the end (warp shuffles, then shared
// memory), so the four global atomics on the same words are made once per block instead of
// once per warp of the lattice.
template <int S, bool PULL>
__global__ void __launch_bounds__(kBX) k_macro_full(const typename Pop<S>::T* __restrict__ fin,
                                                    Grid g, Coef c, float* rho, float* ux,
                                                    float* uy, float* uz,
                                                    unsigned long long* stats) {
    const int nxb = (g.nx + kBX - 1) / kBX;
    const long long segs = (long long)nxb * g.ny * g.nz;
    unsigned int rmin = 0xffffffffu, rmax = 0u, u2max = 0u;
    unsigned int bad = 0;
    for (long long t = blockIdx.x; t < segs; t += gridDim.x) {
        const int x = (int)(t % nxb) * kBX + threadIdx.x;
        const long long row = t / nxb;
        const int y = (int)(row % g.ny), z = (int)(row / g.ny);
        if (x >= g.nx) continue;
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
        const float u = mx / r, v = my / r, w = mz / r;
        const long long cell = (row * g.pitch) + x;
        rho[cell] = r;
        ux[cell] = u;
        uy[cell] = v;
        uz[cell] = w;
        if (stats) {
            const float u2 = u * u + v * v + w * w;
            if (!isfinite(r) || !isfinite(u2)) {
                bad += 1;
            } else {
                rmin = min(rmin, ordered(r));
                rmax = max(rmax, ordered(r));
                u2max = max(u2max, ordered(u2));
            }
        }
    }
    if (!stats) return;
    for (int o = 16; o > 0; o >>= 1) {
        rmin = min(rmin, __shfl_xor_sync(0xffffffffu, rmin, o));
        rmax = max(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        u2max = max(u2max, __shfl_xor_sync(0xffffffffu, u2max, o));
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    __shared__ unsigned int red[kBX / 32][4];
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        red[warp][0] = rmin; red[warp][1] = rmax; red[warp][2] = u2max; red[warp][3] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kBX / 32; ++k) {
            rmin = min(rmin, red[k][0]);
            rmax = max(rmax, red[k][1]);
            u2max = max(u2max, red[k][2]);
            bad += red[k][3];
        }
        if (rmin != 0xffffffffu) {
            atomicMin(stats + 0, (unsigned long long)rmin);
            atomicMax(stats + 1, (unsigned long long)rmax);
            atomicMax(stats + 2, (unsigned long long)u2max);
        }
        if (bad) atomicAdd(stats + 3, (unsigned long long)bad);
    }
}

// Tiled transpose between the padded (z, y, x) layout and the reference (x, y, z) layout.
constexpr int kT = 32;

__device__ __forceinline__ float as_force(float v) { return v; }
__device__ __forceinline__ float as_force(long long v) { return qforce(v); }

template <typename T>
__global__ void k_export_field(const T* __restrict__ a, float* __restrict__ out, Grid g,
                               float clipv) {
    __shared__ float tile[kT][kT + 1];
    const int x0 = blockIdx.x * kT, z0 = blockIdx.z * kT, y = blockIdx.y;
    for (int r = threadIdx.y; r < kT; r += blockDim.y) {
        const int z = z0 + r, x = x0 + threadIdx.x;
        float v = 0.f;
        if (z < g.nz && x < g.nx) v = as_force(a[((long long)z * g.ny + y) * g.pitch + x]);
        if (clipv > 0.f) v = fminf(fmaxf(v, -clipv), clipv);
        tile[r][threadIdx.x] = v;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < kT; r += blockDim.y) {
        const int x = x0 + r, z = z0 + threadIdx.x;
        if (x < g.nx && z < g.nz) out[((long long)x * g.ny + y) * g.nz + z] = tile[threadIdx.x][r];
    }
}

__global__ void k_import_field(const float* __restrict__ in, float* __restrict__ a, Grid g) {
    __shared__ float tile[kT][kT + 1];
    const int x0 = blockIdx.x * kT, z0 = blockIdx.z * kT, y = blockIdx.y;
    for (int r = threadIdx.y; r < kT; r += blockDim.y) {
        const int x = x0 + r, z = z0 + threadIdx.x;
        float v = 0.f;
        if (x < g.nx && z < g.nz) v = in[((long long)x * g.ny + y) * g.nz + z];
        tile[threadIdx.x][r] = v;
    }
    __syncthreads();
    for (int r = threadIdx.y; r < kT; r += blockDim.y) {
        const int z = z0 + r, x = x0 + threadIdx.x;
        if (z < g.nz && x < g.nx) a[((long long)z * g.ny + y) * g.pitch + x] = tile[r][threadIdx.x];
    }
}

template <int S, bool PULL>
__global__ void k_export_populations(const typename Pop<S>::T* __restrict__ fin, float* out,
                                     Grid g, Coef c) {
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    float f[19];
    gather<S, PULL>(fin, g, c, x, y, z, f);
    float* o = out + (((long long)x * g.ny + y) * g.nz + z) * 19;
#pragma unroll
    for (int q = 0; q < 19; ++q) o[q] = f[q];
}

template <int S>
__global__ void k_import_populations(const float* __restrict__ in, typename Pop<S>::T* f,
                                     Grid g) {
    const int x = blockIdx.x * kBX + threadIdx.x;
    const int y = blockIdx.y, z = blockIdx.z;
    if (x >= g.nx) return;
    const float* i = in + (((long long)x * g.ny + y) * g.nz + z) * 19;
    const long long cell = ((long long)z * g.ny + y) * g.pitch + x;
#pragma unroll
    for (int q = 0; q < 19; ++q) Pop<S>::st(f + q * g.plane + cell, q, i[q]);
}

// z-vorticity of one z plane as the reference's renderers take it (render_2d.py:272-275,
// fish/main_fish.py:308-309): w = d(ux)/dy - d(uy)/dx with NumPy gradient rules, central
// differences inside and one-sided first differences on the edges (unit spacing);
// output (Nx, Ny), y fastest.
__global__ void k_vorticity_slice(const float* __restrict__ ux, const float* __restrict__ uy,
                                  Grid g, int z, float* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= g.nx) return;
    const long long row = (long long)z * g.ny * g.pitch;
    auto at = [&](const float* a, int xx, int yy) { return a[row + (long long)yy * g.pitch + xx]; };
    float dux_dy, duy_dx;
    if (g.ny == 1) dux_dy = 0.f;
    else if (y == 0) dux_dy = at(ux, x, 1) - at(ux, x, 0);
    else if (y == g.ny - 1) dux_dy = at(ux, x, y) - at(ux, x, y - 1);
    else dux_dy = 0.5f * (at(ux, x, y + 1) - at(ux, x, y - 1));
    if (x == 0) duy_dx = at(uy, 1, y) - at(uy, 0, y);
    else if (x == g.nx - 1) duy_dx = at(uy, x, y) - at(uy, x - 1, y);
    else duy_dx = 0.5f * (at(uy, x + 1, y) - at(uy, x - 1, y));
    out[(long long)x * g.ny + y] = dux_dy - duy_dx;
}

void launch_vorticity_slice(const float* ux, const float* uy, const Grid& g, int z, float* out,
                            cudaStream_t st) {
    k_vorticity_slice<<<dim3((g.nx + 127) / 128, g.ny), 128, 0, st>>>(ux, uy, g, z, out);
}

// rho = 1, u = (ux_in, uy_in, 0): the macro fields _init_feq sets (clbm_moving.py:88-91)
__global__ void k_fill_macro(Grid g, Coef c, float* rho, float* ux, float* uy, float* uz) {
    const int x = blockIdx.x * kBX + threadIdx.x;
    if (x >= g.nx) return;
    const long long cell = ((long long)blockIdx.z * g.ny + blockIdx.y) * g.pitch + x;
    rho[cell] = 1.0f;
    ux[cell] = c.ux_in;
    uy[cell] = c.uy_in;
    uz[cell] = 0.0f;
}

// ---------------------------------------------------------------- launchers
static dim3 cell_grid(const Grid& g) { return dim3((g.nx + kBX - 1) / kBX, g.ny, g.nz); }

// Blocks of the grid-stride macro pass: 16 resident blocks of kBX threads per SM.
static int macro_full_blocks() {
    static int n = 0;
    if (n == 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
            sms = 148;
        n = sms * 16;
    }
    return n;
}

#define CLBM_DISPATCH_STORE(storage, ...)                                                  \
    switch (storage) {                                                                     \
        case CLBM_STORE_F32: { constexpr int S_ = CLBM_STORE_F32; __VA_ARGS__; } break;   \
        case CLBM_STORE_F16S: { constexpr int S_ = CLBM_STORE_F16S; __VA_ARGS__; } break; \
        default: { constexpr int S_ = CLBM_STORE_BF16S; __VA_ARGS__; } break;             \
    }

// Bounds-check self test: one index test just past the end of the populations (no access),
// which in the bounds-checked build sets kStatusBounds.
__global__ void k_bounds_selftest(Grid g) {
    if (threadIdx.x == 0) (void)in_bounds(19LL * g.plane, 19LL * g.plane, g.status);
}

void launch_bounds_selftest(const Grid& g, cudaStream_t st) { k_bounds_selftest<<<1, 32, 0, st>>>(g); }

// Architecture the bulk stream-collide kernel was compiled for, as the CUDA runtime reports
// it (major * 10 + minor of the SASS it loaded), and its PTX version.
cudaError_t stream_collide_binary_version(int* binary, int* ptx) {
    cudaFuncAttributes fa{};
    const cudaError_t err = cudaFuncGetAttributes(&fa, k_stream_collide<CLBM_STORE_F32, true, kForceSkipBand, true>);
    if (err != cudaSuccess) return err;
    *binary = fa.binaryVersion;
    *ptx = fa.ptxVersion;
    return cudaSuccess;
}

void launch_init(int storage, void* f, const Grid& g, const Coef& c, cudaStream_t st) {
    CLBM_DISPATCH_STORE(storage, (k_init<S_><<<cell_grid(g), kBX, 0, st>>>(
                                     (typename Pop<S_>::T*)f, g, c)));
}

template <int S, bool PULL, int FMODE>
static void tma_launch(const void* fin, void* fout, const Grid& g, const Coef& c,
                       const ForceArgs& fa, cudaStream_t st) {
    using T = typename Stg<S>::T;
    const dim3 grid((g.nx + g.seg - 1) / g.seg, g.ny, g.nz);
    const size_t smem = (size_t)19 * (g.seg + 2 * kHalo) * sizeof(T);
    k_stream_collide_tma<S, PULL, FMODE><<<grid, g.seg / 2, smem, st>>>((const T*)fin, (T*)fout, g, c, fa);
}

template <int S, bool PULL, bool IDX32>
static void cell_launch(int fmode, const void* fin, void* fout, const Grid& g, const Coef& c,
                        const ForceArgs& fa, cudaStream_t st) {
    using T = typename Pop<S>::T;
    if (fmode == kForceNone)
        k_stream_collide<S, PULL, kForceNone, IDX32><<<cell_grid(g), kBX, 0, st>>>((const T*)fin, (T*)fout, g, c, fa);
    else if (fmode == kForceBand)
        k_stream_collide<S, PULL, kForceBand, IDX32><<<cell_grid(g), kBX, 0, st>>>((const T*)fin, (T*)fout, g, c, fa);
    else if (fmode == kForceSkipBand)
        k_stream_collide<S, PULL, kForceSkipBand, IDX32><<<cell_grid(g), kBX, 0, st>>>((const T*)fin, (T*)fout, g, c, fa);
    else
        k_stream_collide<S, PULL, kForceDense, IDX32><<<cell_grid(g), kBX, 0, st>>>((const T*)fin, (T*)fout, g, c, fa);
}

template <int S, bool PULL>
static void sc_launch(int fmode, int variant, const void* fin, void* fout, const Grid& g,
                      const Coef& c, const ForceArgs& fa, cudaStream_t st) {
    if (variant == kVariantStaged) {
        if (fmode == kForceNone) tma_launch<S, PULL, kForceNone>(fin, fout, g, c, fa, st);
        else if (fmode == kForceBand) tma_launch<S, PULL, kForceBand>(fin, fout, g, c, fa, st);
        else if (fmode == kForceSkipBand) tma_launch<S, PULL, kForceSkipBand>(fin, fout, g, c, fa, st);
        else tma_launch<S, PULL, kForceDense>(fin, fout, g, c, fa, st);
        return;
    }
    if constexpr (S != CLBM_STORE_F32) if (variant == kVariantPair) {
        const int px = pair_threads(g.nx);
        if (px == 64) pair_launch<S, PULL, 64>(fmode, fin, fout, g, c, fa, st);
        else if (px == 32) pair_launch<S, PULL, 32>(fmode, fin, fout, g, c, fa, st);
        else pair_launch<S, PULL, 128>(fmode, fin, fout, g, c, fa, st);
        return;
    }
    // 32-bit element indices while every index of the 19 planes fits
    if (19LL * g.plane <= 0xffffffffLL) cell_launch<S, PULL, true>(fmode, fin, fout, g, c, fa, st);
    else cell_launch<S, PULL, false>(fmode, fin, fout, g, c, fa, st);
}

void launch_stream_collide(int storage, bool pull, int fmode, int variant, const void* fin,
                           void* fout, const Grid& g, const Coef& c, const ForceArgs& fa,
                           cudaStream_t st) {
    CLBM_DISPATCH_STORE(storage, {
        if (pull) sc_launch<S_, true>(fmode, variant, fin, fout, g, c, fa, st);
        else sc_launch<S_, false>(fmode, variant, fin, fout, g, c, fa, st);
    });
}

int knob(const char* name, int def) {
    const char* e = std::getenv(name);
    return e ? std::atoi(e) : def;
}

// Launch of the box pass by rows for a box of at most max_bx x max_by x max_bz cells: one
// block per work item of the largest box, at most 4 blocks per SM (then grid-stride).
template <bool SUMS>
static void box_rows_launch(int storage, bool pull, const void* fin, void* fout, const Grid& g,
                            const Coef& c, const ForceArgs& fa, const IbmArrays& a, int max_bx,
                            int max_by, int max_bz, cudaStream_t st) {
    const long long rows = (long long)std::max(max_by, 1) * std::max(max_bz, 1);
    const bool f32 = storage == CLBM_STORE_F32;
    // float32 one cell per thread; the 16-bit pairs start at i0 rounded down to even
    const long long nseg = f32 ? (max_bx + kBoxBlock - 1) / kBoxBlock
                               : (max_bx + 1 + 2 * kBoxBlock - 1) / (2 * kBoxBlock);
    const int blocks = (int)std::max<long long>(1, std::min<long long>(std::max<long long>(nseg, 1) * rows, 4 * 152));
    if (f32) {
        if (pull) k_box_rows_cell<CLBM_STORE_F32, true, SUMS><<<blocks, kBoxBlock, 0, st>>>((const float*)fin, (float*)fout, g, c, fa, a);
        else k_box_rows_cell<CLBM_STORE_F32, false, SUMS><<<blocks, kBoxBlock, 0, st>>>((const float*)fin, (float*)fout, g, c, fa, a);
        return;
    }
    const bool i32 = 19LL * g.plane <= 0xffffffffLL;
#define CLBM_BOX_ROWS(S_)                                                                                  \
    {                                                                                                      \
        using T = typename Pair<S_>::T;                                                                    \
        if (pull && i32) k_box_rows_pair<S_, true, SUMS, true><<<blocks, kBoxBlock, 0, st>>>((const T*)fin, (T*)fout, g, c, fa, a);   \
        else if (pull) k_box_rows_pair<S_, true, SUMS, false><<<blocks, kBoxBlock, 0, st>>>((const T*)fin, (T*)fout, g, c, fa, a);  \
        else if (i32) k_box_rows_pair<S_, false, SUMS, true><<<blocks, kBoxBlock, 0, st>>>((const T*)fin, (T*)fout, g, c, fa, a);  \
        else k_box_rows_pair<S_, false, SUMS, false><<<blocks, kBoxBlock, 0, st>>>((const T*)fin, (T*)fout, g, c, fa, a);          \
    }
    if (storage == CLBM_STORE_F16S) CLBM_BOX_ROWS(CLBM_STORE_F16S)
    else CLBM_BOX_ROWS(CLBM_STORE_BF16S)
#undef CLBM_BOX_ROWS
}

void launch_stream_collide_box(int storage, bool pull, const void* fin, void* fout,
                               const Grid& g, const Coef& c, const ForceArgs& fa, int max_bx,
                               int max_by, int max_bz, cudaStream_t st) {
    box_rows_launch<false>(storage, pull, fin, fout, g, c, fa, IbmArrays{}, max_bx, max_by, max_bz, st);
}

void launch_stream_collide_box_sums(int storage, bool pull, const void* fin, void* fout,
                                    const Grid& g, const Coef& c, const ForceArgs& fa,
                                    const IbmArrays& a, cudaStream_t st) {
    box_rows_launch<true>(storage, pull, fin, fout, g, c, fa, a, a.max_bx, a.max_by, a.max_bz, st);
}

// Blocks of kBoxBlock threads for a box of at most max_cells cells: one cell per thread,
// at most 16 blocks per SM (then grid-stride).
static int box_blocks(long long max_cells) {
    const long long b = (max_cells + kBoxBlock - 1) / kBoxBlock;
    return (int)std::max<long long>(1, std::min<long long>(b, 16 * 152));
}

void launch_macro_full(int storage, bool pull, const void* f, const Grid& g, const Coef& c,
                       float* rho, float* ux, float* uy, float* uz,
                       unsigned long long* stats, cudaStream_t st) {
    CLBM_DISPATCH_STORE(storage, {
        using T = typename Pop<S_>::T;
        const long long segs = (long long)((g.nx + kBX - 1) / kBX) * g.ny * g.nz;
        const int blocks = (int)std::min<long long>(segs, macro_full_blocks());
        if (pull) k_macro_full<S_, true><<<blocks, kBX, 0, st>>>((const T*)f, g, c, rho, ux, uy, uz, stats);
        else k_macro_full<S_, false><<<blocks, kBX, 0, st>>>((const T*)f, g, c, rho, ux, uy, uz, stats);
    });
}

void launch_fill_macro(const Grid& g, const Coef& c, float* rho, float* ux, float* uy,
                       float* uz, cudaStream_t st) {
    k_fill_macro<<<cell_grid(g), kBX, 0, st>>>(g, c, rho, ux, uy, uz);
}

void launch_export_field(const float* a, float* out, const Grid& g, float clipv,
                         cudaStream_t st) {
    dim3 grid((g.nx + kT - 1) / kT, g.ny, (g.nz + kT - 1) / kT);
    k_export_field<float><<<grid, dim3(kT, 8), 0, st>>>(a, out, g, clipv);
}

void launch_export_qfield(const long long* a, float* out, const Grid& g, float clipv,
                          cudaStream_t st) {
    dim3 grid((g.nx + kT - 1) / kT, g.ny, (g.nz + kT - 1) / kT);
    k_export_field<long long><<<grid, dim3(kT, 8), 0, st>>>(a, out, g, clipv);
}

void launch_import_field(const float* in, float* a, const Grid& g, cudaStream_t st) {
    dim3 grid((g.nx + kT - 1) / kT, g.ny, (g.nz + kT - 1) / kT);
    k_import_field<<<grid, dim3(kT, 8), 0, st>>>(in, a, g);
}

void launch_export_populations(int storage, bool pull, const void* f, float* out,
                               const Grid& g, const Coef& c, cudaStream_t st) {
    CLBM_DISPATCH_STORE(storage, {
        using T = typename Pop<S_>::T;
        if (pull) k_export_populations<S_, true><<<cell_grid(g), kBX, 0, st>>>((const T*)f, out, g, c);
        else k_export_populations<S_, false><<<cell_grid(g), kBX, 0, st>>>((const T*)f, out, g, c);
    });
}

void launch_import_populations(int storage, const float* in, void* f, const Grid& g,
                               cudaStream_t st) {
    CLBM_DISPATCH_STORE(storage, {
        using T = typename Pop<S_>::T;
        k_import_populations<S_><<<cell_grid(g), kBX, 0, st>>>(in, (T*)f, g);
    });
}

// Band-prepare needs the same gather; the IBM translation unit calls this launcher.
template <int S, bool PULL>
__global__ void __launch_bounds__(kBoxBlock) k_band_prepare(const typename Pop<S>::T* __restrict__ fin, Grid g, Coef c,
                               IbmDev* dev, long long* fx, long long* fy, float* rho, float* ux,
                               float* uy, float* uz, bool compute_macro) {
    band_prepare_body<S, PULL>(fin, g, c, dev, fx, fy, rho, ux, uy, uz, compute_macro, blockIdx.x,
                               gridDim.x);
}

void launch_band_prepare(int storage, bool pull, const void* f, const Grid& g, const Coef& c,
                         IbmDev* dev, long long* fx, long long* fy, float* rho, float* ux, float* uy,
                         float* uz, int max_bx, int max_by, int max_bz, bool compute_macro,
                         cudaStream_t st) {
    const int blocks = box_blocks((long long)max_bx * max_by * max_bz);
    CLBM_DISPATCH_STORE(storage, {
        using T = typename Pop<S_>::T;
        if (pull) k_band_prepare<S_, true><<<blocks, kBoxBlock, 0, st>>>((const T*)f, g, c, dev, fx, fy, rho, ux, uy, uz, compute_macro);
        else k_band_prepare<S_, false><<<blocks, kBoxBlock, 0, st>>>((const T*)f, g, c, dev, fx, fy, rho, ux, uy, uz, compute_macro);
    });
}

}  // namespace clbm
