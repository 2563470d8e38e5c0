// closure.cu -- learned sub-grid closure: fused stream-collide with the network evaluated
// on the tensor cores, training-sample extraction from box-filtered fine-lattice fields,
// and the training kernels (forward, backward and weight gradients on the tensor cores,
// deterministic reductions, Adam).
//
// The network maps the 19 normalised non-equilibrium central moments of a cell to one
// relaxation rate (th = tanh(z3)):
//   mode 0, higher-order rate (the reference fixes s_q = s_pi = 1, clbm_moving.py:186-194):
//     k3* = (1 - s_h) k3,  k4* = r/9 + (1 - s_h)(k4 - r/9),  s_h = 1 + span th;
//   mode 1, eddy viscosity: the deviatoric second-order moments relax with
//     s_eff = 1 / (1/2 + 3 nu 2^(span g)), g = th (th >= 0) or th / 20 (th < 0), instead of
//     s_v (nu the solver's viscosity): the network adds an eddy viscosity nu_t, trained
//     against the sub-grid stress of the box-filtered fine velocity, tau = -2 nu_t S.
// Dense layers run as tcgen05 MMAs (BF16 operands from shared memory, FP32 accumulators in
// tensor memory, M = 128 rows = one cell or sample per thread of a 128-thread block).
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "closure_device.cuh"

namespace clbm {
using namespace closure;

// ------------------------------------------------------------------ weight images
// BF16 images of W1 [out][in], W2 [out][in] and W2^T [in][out], each 32 x 32 in the
// K-major core-matrix layout (the B operands of the forward and input-gradient MMAs).
__global__ void k_closure_images(const float* __restrict__ p, uint16_t* __restrict__ img) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= kImgElems) return;
    const int which = t >> 10, e = t & 1023, n = e >> 5, k = e & 31;
    const float v = which == 0 ? p[kW1 + n * 32 + k] : which == 1 ? p[kW2 + n * 32 + k] : p[kW2 + k * 32 + n];
    img[which * 1024 + (tc::kmajor_offset(n, k, 32) >> 1)] = bf16_bits(v);
}

void launch_closure_images(const float* params, uint16_t* img, cudaStream_t st) {
    k_closure_images<<<(kImgElems + 255) / 256, 256, 0, st>>>(params, img);
}

namespace {

constexpr uint32_t kIdescFwd = tc::idesc_bf16(128, 32);
constexpr uint32_t kIdescF16 = tc::idesc_f16(128, 32);

// Issue D = A (128 x 32, K-major) * B^T (32 x 32) as two K = 16 MMAs; commit to `bar`
// (the completion of every MMA this thread issued so far) unless it is null.
__device__ __forceinline__ void mma_k32(uint32_t tmem, uint32_t a, uint32_t b, uint64_t* bar,
                                        uint32_t idesc = kIdescFwd) {
    tc::mma(tmem, tc::smem_desc(a, 128, 512), tc::smem_desc(b, 128, 512), idesc, false);
    tc::mma(tmem, tc::smem_desc(a + 256, 128, 512), tc::smem_desc(b + 256, 128, 512), idesc, true);
    if (bar) tc::commit(bar);
}

// 16-bit bits of x in the storage form's own type (FP16 or BF16); exact for the stored
// deviations, which already are values of that type.
template <int S>
__device__ __forceinline__ uint16_t store_bits(float x) {
    if constexpr (S == CLBM_STORE_F16S) return __half_as_ushort(__float2half_rn(x));
    else return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}

// Row `row` of a K-major tile with 32 columns: the 19 values in the storage form's type,
// zeros after them.
template <int S>
__device__ __forceinline__ void put_row19_store(unsigned char* tile, int row, const float (&v)[19]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        uint32_t wv[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int k = 8 * j + 2 * t;
            const uint32_t lo = k < 19 ? store_bits<S>(v[k < 19 ? k : 0]) : 0u;
            const uint32_t hi = k + 1 < 19 ? store_bits<S>(v[k + 1 < 19 ? k + 1 : 0]) : 0u;
            wv[t] = lo | (hi << 16);
        }
        *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(row, 8 * j, 32)) =
            make_uint4(wv[0], wv[1], wv[2], wv[3]);
    }
}

// Block-wide barrier that also orders tensor-core work around it.
__device__ __forceinline__ void tc_sync() {
    tc::fence_smem_async();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
}

}  // namespace

// ------------------------------------------------------------------ fused inference
// Persistent stream-collide pass with the closure: 128 threads, one cell each; a block
// takes tiles of 128 consecutive cells (x fastest across row ends). Per tile: gather,
// moments and features (row of the A tile), layer 1 MMA, GELU, layer 2 MMA, GELU, output
// layer on the CUDA cores, collision with s_h, store. Cells of the IBM force box (SkipBand)
// are left to the box pass, which uses the plain collision with forcing; the inlet and
// outlet columns (x = 0, nx - 1) keep the plain rates.
// FMMA (16-bit forms): the raw moments of the features come from one more MMA per tile,
// D = H M_raw^T with H the 128 cells' 19 stored deviations (exact in the storage type, FP16
// or BF16) and M_raw's entries 0, +-1 (exact), FP32 accumulation; the binomial shift to
// central moments (per-cell velocity) stays on the CUDA cores.
template <int S, bool PULL, int FMODE, bool IDX32, bool FMMA>
__global__ void __launch_bounds__(128, 8) k_closure_stream_collide(const typename Pop<S>::T* __restrict__ fin,
                                                                typename Pop<S>::T* __restrict__ fout,
                                                                Grid g, Coef c, ForceArgs fa,
                                                                ClosureArgs ca) {
    constexpr bool DEV = Pop<S>::kShifted;
    static_assert(!FMMA || DEV, "the feature MMA takes the 16-bit stored deviations");
    __shared__ __align__(1024) unsigned char sA[128 * 32 * 2];
    __shared__ __align__(1024) unsigned char sW[(FMMA ? 3 : 2) * 32 * 32 * 2];
    __shared__ NetSmem net;
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < (2 * 32 * 32 * 2) / 16; i += 128)
        reinterpret_cast<uint4*>(sW)[i] = reinterpret_cast<const uint4*>(ca.img)[i];
    if (FMMA) {
        // B of the feature MMA: M_raw as [moment][population], 32 x 32, K-major
        for (int e = tid; e < 32 * 32; e += 128) {
            const int n = e >> 5, k = e & 31;
            const int v = (n < kIn && k < 19) ? mraw_entry(n, k) : 0;
            *reinterpret_cast<uint16_t*>(sW + 4096 + tc::kmajor_offset(n, k, 32)) =
                v == 0 ? (uint16_t)0 : store_bits<S>((float)v);
        }
    }
    load_net(ca.params, net, tid, 128);
    if (warp == 0) tc::alloc(&tbase, 32);
    if (tid == 0) tc::bar_init(&bar, 1);
    tc_sync();
    const uint32_t tm = tbase;
    const uint32_t aA = tc::smem_addr(sA), aW1 = tc::smem_addr(sW), aW2 = aW1 + 2048, aM = aW1 + 4096;
    const float nu = (1.0f / (1.0f - c.one_m_sv) - 0.5f) * (1.0f / 3.0f);  // solver viscosity
    uint32_t phase = 0;
    bool ok = true;
    const Band band = (FMODE == kForceSkipBand) ? load_band(fa.dev, fa.slot)
                                                : Band{};
    for (long long tile = blockIdx.x; tile < ca.tiles; tile += gridDim.x) {
        const long long i = tile * 128 + tid;
        bool use = i < ca.cells;
        int x = 0, y = 0, z = 0;
        if (use) {
            if (ca.cells <= 0xffffffffLL) {   // 32-bit divisions (64-bit ones are far slower)
                const unsigned ui = (unsigned)i, row = ui / (unsigned)g.nx;
                x = (int)(ui - row * (unsigned)g.nx);
                y = (int)(row % (unsigned)g.ny);
                z = (int)(row / (unsigned)g.ny);
            } else {
                const long long row = i / g.nx;
                x = (int)(i - row * g.nx);
                y = (int)(row % g.ny);
                z = (int)(row / g.ny);
            }
            if (FMODE == kForceSkipBand && in_band(band, x, y, z, g.ny, g.nz)) use = false;
        }
        float f[19];
        float v[32];
        bool w = true;
        if (FMMA) {
            if (use) {
                gather<S, PULL, true, IDX32>(fin, g, c, x, y, z, f);
            } else {
#pragma unroll
                for (int q = 0; q < 19; ++q) f[q] = 0.0f;
            }
            put_row19_store<S>(sA, tid, f);
            tc_sync();
            if (tid == 0) {
                mma_k32(tm, aA, aM, &bar, S == CLBM_STORE_F16S ? kIdescF16 : kIdescFwd);
                w = tc::bar_wait(&bar, phase, g.spin_limit);
            }
            ok = !__syncthreads_or(!w);
            phase ^= 1;
            if (!ok) break;
            tc::fence_after();
            tc::ld32(tc::lane_addr(tm, warp, 0), v);
            if (use) {
                CMom m;
                moments_from_mraw(v, m);
                standardise(m, net, v);
            } else {
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = 0.0f;
            }
            // every thread has read its row of the feature result before the A tile and
            // the accumulator are reused
            tc::fence_before();
            __syncthreads();
            tc::fence_after();
        } else if (use) {
            gather<S, PULL, true, IDX32>(fin, g, c, x, y, z, f);
            CMom m;
            moments_full<DEV>(f, m);
            standardise(m, net, v);
        } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] = 0.0f;
        }
        put_row32(sA, tid, v);
        tc_sync();
        // one thread issues the MMAs and waits for them; the barrier releases the block
        if (tid == 0) {
            mma_k32(tm, aA, aW1, &bar);
            w = tc::bar_wait(&bar, phase, g.spin_limit);
        }
        ok = !__syncthreads_or(!w);
        phase ^= 1;
        if (!ok) break;
        tc::fence_after();
        tc::ld32(tc::lane_addr(tm, warp, 0), v);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const float2 b = reinterpret_cast<const float2*>(net.b1)[j];
            const float2 h = vunpack(gelu2(vpack(v[2 * j], v[2 * j + 1]) + vpack(b.x, b.y)));
            v[2 * j] = h.x;
            v[2 * j + 1] = h.y;
        }
        put_row32(sA, tid, v);
        tc_sync();
        if (tid == 0) {
            mma_k32(tm, aA, aW2, &bar);
            w = tc::bar_wait(&bar, phase, g.spin_limit);
        }
        ok = !__syncthreads_or(!w);
        phase ^= 1;
        if (!ok) break;
        tc::fence_after();
        tc::ld32(tc::lane_addr(tm, warp, 0), v);
        V2 acc = vsplat(0.0f, V2{});
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const float2 b = reinterpret_cast<const float2*>(net.b2)[j];
            const float2 w3 = reinterpret_cast<const float2*>(net.w3)[j];
            acc = vfma(vpack(w3.x, w3.y), gelu2(vpack(v[2 * j], v[2 * j + 1]) + vpack(b.x, b.y)), acc);
        }
        const float2 accs = vunpack(acc);
        const float z3 = net.b3 + (accs.x + accs.y);
        // inlet and outlet columns keep the plain rates (no training samples there)
        const bool edge = x == 0 || x == g.nx - 1;
        if (use) {
            const float th = tanh_approx(z3);
            if (net.mode == 1) {
                const float se = edge ? 1.0f - c.one_m_sv : eddy_rate(nu, net.span, th);
                collide_sv<DEV>(f, c, 1.0f - se);
            } else {
                const float sh = edge ? 1.0f : 1.0f + net.span * th;
                CMom m;  // recomputed rather than kept live across the network
                moments_full<DEV>(f, m);
                float ho[9];
                higher_order_post(m, sh, ho);
                collide_ho<DEV>(f, c, ho);
            }
            store_raw<S, IDX32>(fout, g, ((long long)z * g.ny + y) * g.pitch + x, f);
        }
    }
    if (!ok) {
        if (tid == 0) atomicOr(g.status, kStatusWaitTimeout);
        tc::bar_wait(&bar, phase ^ 1, g.spin_limit);  // the MMA that did not report in time
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) tc::dealloc(tm, 32);
}

#define CLBM_CL_STORE(storage, ...)                                                          \
    switch (storage) {                                                                       \
        case CLBM_STORE_F32: { constexpr int S_ = CLBM_STORE_F32; __VA_ARGS__; } break;     \
        case CLBM_STORE_F16S: { constexpr int S_ = CLBM_STORE_F16S; __VA_ARGS__; } break;   \
        default: { constexpr int S_ = CLBM_STORE_BF16S; __VA_ARGS__; } break;               \
    }

// Feature path of the fused closure pass (16-bit forms): CLBM_CLOSURE_FEATURES=mma takes
// the raw moments from the tensor cores, =cores (default) from the CUDA cores.
static bool closure_features_mma(int storage) {
    if (storage == CLBM_STORE_F32) return false;
    const char* e = std::getenv("CLBM_CLOSURE_FEATURES");   // read at every launch
    return e && !std::strcmp(e, "mma");
}

template <int S, bool PULL, bool FMMA>
static void closure_sc_f(int fmode, const void* fin, void* fout, const Grid& g, const Coef& c,
                         const ForceArgs& fa, const ClosureArgs& ca, int grid, cudaStream_t st) {
    using T = typename Pop<S>::T;
    if (19LL * g.plane <= 0xffffffffLL) {   // every element index fits 32 bits
        if (fmode == kForceSkipBand)
            k_closure_stream_collide<S, PULL, kForceSkipBand, true, FMMA><<<grid, 128, 0, st>>>((const T*)fin, (T*)fout, g, c, fa, ca);
        else
            k_closure_stream_collide<S, PULL, kForceNone, true, FMMA><<<grid, 128, 0, st>>>((const T*)fin, (T*)fout, g, c, fa, ca);
        return;
    }
    if (fmode == kForceSkipBand)
        k_closure_stream_collide<S, PULL, kForceSkipBand, false, FMMA><<<grid, 128, 0, st>>>((const T*)fin, (T*)fout, g, c, fa, ca);
    else
        k_closure_stream_collide<S, PULL, kForceNone, false, FMMA><<<grid, 128, 0, st>>>((const T*)fin, (T*)fout, g, c, fa, ca);
}

template <int S, bool PULL>
static void closure_sc(int fmode, const void* fin, void* fout, const Grid& g, const Coef& c,
                       const ForceArgs& fa, const ClosureArgs& ca, int grid, cudaStream_t st) {
    if constexpr (S != CLBM_STORE_F32) {
        if (closure_features_mma(S)) {
            closure_sc_f<S, PULL, true>(fmode, fin, fout, g, c, fa, ca, grid, st);
            return;
        }
    }
    closure_sc_f<S, PULL, false>(fmode, fin, fout, g, c, fa, ca, grid, st);
}

// Persistent grid: the blocks that fit on an SM by registers (65,536 per SM) and by
// tensor memory (32 of 512 columns per block), times the SM count.
int closure_grid(int storage) {
    int dev = 0, sms = 0, regs = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncAttributes fa{};
    CLBM_CL_STORE(storage, {
        int r0 = 0, r1 = 0;
        if (cudaFuncGetAttributes(&fa, k_closure_stream_collide<S_, true, kForceSkipBand, true, false>) == cudaSuccess)
            r0 = fa.numRegs;
        if constexpr (S_ != CLBM_STORE_F32)
            if (cudaFuncGetAttributes(&fa, k_closure_stream_collide<S_, true, kForceSkipBand, true, true>) == cudaSuccess)
                r1 = fa.numRegs;
        regs = std::max(r0, r1);
    });
    cudaGetLastError();
    const int per_regs = regs > 0 ? 65536 / (128 * ((regs + 7) / 8 * 8)) : 4;
    const int per = std::min(std::max(per_regs, 1), 16);
    return std::max(sms, 1) * per;
}

void launch_closure_stream_collide(int storage, bool pull, int fmode, const void* fin, void* fout,
                                   const Grid& g, const Coef& c, const ForceArgs& fa,
                                   const ClosureArgs& cargs, int grid, cudaStream_t st) {
    ClosureArgs ca = cargs;
    ca.tiles = (ca.cells + 127) / 128;
    CLBM_CL_STORE(storage, {
        if (pull) closure_sc<S_, true>(fmode, fin, fout, g, c, fa, ca, grid, st);
        else closure_sc<S_, false>(fmode, fin, fout, g, c, fa, ca, grid, st);
    });
}

// ------------------------------------------------------------------ training samples
// Box filter of a fine lattice twice as fine in each direction: coarse cell (I, J, K) gets
// the mean of the post-stream (pre-collision) populations of fine cells (2I + a, 2J + b,
// 2K + c), a, b, c in {0, 1} (planes 0-18 of `out`), and the means of the fine velocity
// u = m / rho and of its products u_i u_j (planes 19-21: ux, uy, uz; 22-27: xx, yy, zz,
// xy, xz, yz). Float32 fine storage.
template <bool PULL>
__global__ void __launch_bounds__(128) k_filter2(const float* __restrict__ ff, Grid gf, Coef cf,
                                                 float* __restrict__ out, Grid gc) {
    const int X = blockIdx.x * 128 + threadIdx.x, Y = blockIdx.y, Z = blockIdx.z;
    if (X >= gc.nx) return;
    float acc[19], aux[kAux];
#pragma unroll
    for (int q = 0; q < 19; ++q) acc[q] = 0.0f;
#pragma unroll
    for (int i = 0; i < kAux; ++i) aux[i] = 0.0f;
    for (int s = 0; s < 8; ++s) {
        float v[19];
        gather<CLBM_STORE_F32, PULL, false>(ff, gf, cf, 2 * X + (s & 1), 2 * Y + ((s >> 1) & 1),
                                            2 * Z + (s >> 2), v);
        float r = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
#pragma unroll
        for (int q = 0; q < 19; ++q) {
            acc[q] += v[q];
            r += v[q];
            mx += (float)ex(q) * v[q];
            my += (float)ey(q) * v[q];
            mz += (float)ez(q) * v[q];
        }
        const float u = mx / r, w = mz / r, vv = my / r;
        aux[0] += u; aux[1] += vv; aux[2] += w;
        aux[3] += u * u; aux[4] += vv * vv; aux[5] += w * w;
        aux[6] += u * vv; aux[7] += u * w; aux[8] += vv * w;
    }
    const long long cell = ((long long)Z * gc.ny + Y) * gc.pitch + X;
#pragma unroll
    for (int q = 0; q < 19; ++q) out[q * gc.plane + cell] = 0.125f * acc[q];
#pragma unroll
    for (int i = 0; i < kAux; ++i) out[(19 + i) * gc.plane + cell] = 0.125f * aux[i];
}

void launch_filter2(bool pull, const float* ff, const Grid& gf, const Coef& cf, float* out,
                    const Grid& gc, cudaStream_t st) {
    const dim3 grid((gc.nx + 127) / 128, gc.ny, gc.nz);
    if (pull) k_filter2<true><<<grid, 128, 0, st>>>(ff, gf, cf, out, gc);
    else k_filter2<false><<<grid, 128, 0, st>>>(ff, gf, cf, out, gc);
}

// Sample j: coarse cell cells[j] (x + nx (y + ny z), 2 <= x <= nx - 3). Features from the
// filtered pre-collision state f0; higher-order targets from the ideal post-collision
// state f*_q(x) = f1_q(x + e_q) (f1 one coarse step later), as central moments about the
// velocity of f0, divided by its density; sub-grid stress targets from the filtered
// velocity fields of f0: tau_ij = <u_i u_j> - <u_i><u_j> at the cell and the strain rate
// S_ij = (d_i <u_j> + d_j <u_i>) / 2 by central differences (y, z periodic). Layout
// samples[i * stride + offset + j]: i < 19 features, 19 <= i < 28 third order then fourth
// order minus rho*/9, 28 <= i < 33 tau and 33 <= i < 38 S, each as (xy, xz, yz, xx - yy,
// xx - zz).
__global__ void k_closure_samples(const float* __restrict__ f0, const float* __restrict__ f1, Grid gc,
                                  const long long* __restrict__ cells, long long n,
                                  float* __restrict__ samples, long long stride, long long offset) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const long long id = cells[j];
    const int x = (int)(id % gc.nx);
    const long long row = id / gc.nx;
    const int y = (int)(row % gc.ny), z = (int)(row / gc.ny);
    const long long cell = ((long long)z * gc.ny + y) * gc.pitch + x;
    const int ym = y == 0 ? gc.ny - 1 : y - 1, yp = y == gc.ny - 1 ? 0 : y + 1;
    const int zm = z == 0 ? gc.nz - 1 : z - 1, zp = z == gc.nz - 1 ? 0 : z + 1;
    auto at = [&](int xx, int yy, int zz) { return ((long long)zz * gc.ny + yy) * gc.pitch + xx; };
    float f[19], fs[19];
#pragma unroll
    for (int q = 0; q < 19; ++q) f[q] = f0[q * gc.plane + cell];
#pragma unroll
    for (int q = 0; q < 19; ++q) {
        const int yy = ey(q) > 0 ? yp : (ey(q) < 0 ? ym : y);
        const int zz = ez(q) > 0 ? zp : (ez(q) < 0 ? zm : z);
        fs[q] = f1[q * gc.plane + at(x + ex(q), yy, zz)];
    }
    CMom m;
    moments_full<false>(f, m);
    const Raw rs = raw_moments<false>(fs);
    float t[kIn];
    central_moments(rs, m.u, m.v, m.w, m.r, t);
    float* out = samples + offset + j;
#pragma unroll
    for (int i = 0; i < kIn; ++i) out[i * stride] = m.x[i];
#pragma unroll
    for (int i = 0; i < kTargets; ++i) out[(kIn + i) * stride] = t[10 + i];
    // sub-grid stress and filtered strain rate
    const float* a = f0 + 19 * gc.plane;  // aux planes
    const float ux = a[cell], uy = a[gc.plane + cell], uz = a[2 * gc.plane + cell];
    const float txx = a[3 * gc.plane + cell] - ux * ux, tyy = a[4 * gc.plane + cell] - uy * uy;
    const float tzz = a[5 * gc.plane + cell] - uz * uz, txy = a[6 * gc.plane + cell] - ux * uy;
    const float txz = a[7 * gc.plane + cell] - ux * uz, tyz = a[8 * gc.plane + cell] - uy * uz;
    auto d = [&](int comp, long long cp, long long cm) {
        return 0.5f * (a[comp * gc.plane + cp] - a[comp * gc.plane + cm]);
    };
    const long long xp_ = at(x + 1, y, z), xm_ = at(x - 1, y, z);
    const long long yp_ = at(x, yp, z), ym_ = at(x, ym, z);
    const long long zp_ = at(x, y, zp), zm_ = at(x, y, zm);
    const float dux_dx = d(0, xp_, xm_), duy_dy = d(1, yp_, ym_), duz_dz = d(2, zp_, zm_);
    const float sxy = 0.5f * (d(0, yp_, ym_) + d(1, xp_, xm_));
    const float sxz = 0.5f * (d(0, zp_, zm_) + d(2, xp_, xm_));
    const float syz = 0.5f * (d(1, zp_, zm_) + d(2, yp_, ym_));
    const float sg[kSgs] = {txy, txz, tyz, txx - tyy, txx - tzz,
                            sxy, sxz, syz, dux_dx - duy_dy, dux_dx - duz_dz};
#pragma unroll
    for (int i = 0; i < kSgs; ++i) out[(kIn + kTargets + i) * stride] = sg[i];
}

void launch_closure_samples(const float* f0, const float* f1, const Grid& gc, const long long* cells,
                            long long n, float* samples, long long stride, long long offset,
                            cudaStream_t st) {
    if (n <= 0) return;
    k_closure_samples<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(f0, f1, gc, cells, n, samples, stride,
                                                                  offset);
}

// Per-block partial sums of the features and their squares over samples [0, n), of the
// squared pre-collision higher-order moments (sum_j x_{10+j}^2) and of the squared
// deviatoric sub-grid stress, for the standardisation and the loss scales; reduced in a
// fixed order by k_stats_final.
__global__ void __launch_bounds__(256) k_sample_stats(const float* __restrict__ s, long long stride,
                                                      long long n, double* __restrict__ part) {
    __shared__ double red[256];
    double acc[kStats];
#pragma unroll
    for (int i = 0; i < kStats; ++i) acc[i] = 0.0;
    for (long long j = (long long)blockIdx.x * 256 + threadIdx.x; j < n; j += (long long)gridDim.x * 256) {
        float xf[kIn];
#pragma unroll
        for (int i = 0; i < kIn; ++i) {
            xf[i] = s[i * stride + j];
            const double v = xf[i];
            acc[i] += v;
            acc[kIn + i] += v * v;
            if (i >= 10) acc[2 * kIn] += v * v;
        }
#pragma unroll
        for (int i = 0; i < kSgs / 2; ++i) {
            const double tv = s[(kIn + kTargets + i) * stride + j];
            acc[2 * kIn + 1] += tv * tv;
        }
    }
    for (int i = 0; i < kStats; ++i) {
        red[threadIdx.x] = acc[i];
        __syncthreads();
        for (int w = 128; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) part[(long long)blockIdx.x * kStats + i] = red[0];
        __syncthreads();
    }
}

__global__ void k_stats_final(const double* __restrict__ part, int blocks, double* __restrict__ out) {
    const int i = threadIdx.x;
    if (i >= kStats) return;
    double a = 0.0;
    for (int b = 0; b < blocks; ++b) a += part[(long long)b * kStats + i];
    out[i] = a;
}

void launch_sample_stats(const float* s, long long stride, long long n, double* part, int blocks,
                         double* out, cudaStream_t st) {
    k_sample_stats<<<blocks, 256, 0, st>>>(s, stride, n, part);
    k_stats_final<<<1, 64, 0, st>>>(part, blocks, out);
}

// ------------------------------------------------------------------ training
// Shared-memory plan of the training kernel (dynamic, 1024-byte aligned):
//   sX   128 x 32   K-major: features, then h1, then delta2 (A of the three 32-wide MMAs)
//   sW   W1, W2, W2^T images (B operands)
//   sAw  128 x 128  K-major over samples: rows 0-31 delta1^T, 32-63 delta2^T, 64 delta3
//   sBw  112 x 128  K-major over samples: rows 0-31 x^T, 32-63 h1^T, 64 ones, 80-111 h2^T
// Weight and bias gradients are one MMA chain per tile, D[128 x 112] += sAw * sBw^T,
// accumulated over the block's tiles in tensor-memory columns 32-143:
//   D[o][n]          o < 32: dW1[o][n] (n < 32), db1[o] (n = 64)
//   D[32 + o][32 + n]        dW2[o][n],          db2[o] (n = 64)
//   D[64][80 + n]            dW3[n],             db3    (n = 64)
constexpr int kTrSX = 0, kTrSW = 8192, kTrAw = kTrSW + 6144, kTrBw = kTrAw + 32768;
constexpr int kTrSmem = kTrBw + 112 * 128 * 2;  // 75,776 bytes
constexpr int kPart = kTrainable + 1;           // gradients, then the loss sum
constexpr uint32_t kIdescW = tc::idesc_bf16(128, 112);

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ void put_col(unsigned char* tile, int row, int col, float v) {
    *reinterpret_cast<uint16_t*>(tile + tc::kmajor_offset(row, col, 128)) = bf16_bits(v);
}

template <bool GRAD>
__global__ void __launch_bounds__(128) k_closure_train(TrainArgs a) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ NetSmem net;
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tbase;
    __shared__ float red[128];
    unsigned char* sX = smem + kTrSX;
    unsigned char* sW = smem + kTrSW;
    unsigned char* sAw = smem + kTrAw;
    unsigned char* sBw = smem + kTrBw;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < 6144 / 16; i += 128)
        reinterpret_cast<uint4*>(sW)[i] = reinterpret_cast<const uint4*>(a.img)[i];
    // zero the weight-gradient operands once (rows that stay zero)
    for (int i = tid; i < (32768 + 112 * 128 * 2) / 16; i += 128)
        reinterpret_cast<uint4*>(sAw)[i] = make_uint4(0, 0, 0, 0);
    load_net(a.params, net, tid, 128);
    if (warp == 0) tc::alloc(&tbase, 256);
    if (tid == 0) tc::bar_init(&bar, 1);
    tc_sync();
    const uint32_t tm = tbase;
    const uint32_t aX = tc::smem_addr(sX), aW1 = tc::smem_addr(sW), aW2 = aW1 + 2048, aW2T = aW1 + 4096;
    const uint32_t aAw = tc::smem_addr(sAw), aBw = tc::smem_addr(sBw);
    uint32_t phase = 0;
    bool ok = true;
    float loss = 0.0f;
    int ntile = 0;
    const long long tiles = (a.batch + 127) / 128;
    for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++ntile) {
        const long long slot = tile * 128 + tid;
        const bool valid = slot < a.batch;
        long long sidx = 0;
        if (valid)
            sidx = a.random ? a.off + (long long)(mix64(a.seed ^ (unsigned long long)slot) % (unsigned long long)a.count)
                            : a.off + slot;
        float x[kIn], tg[kSgs];
#pragma unroll
        for (int i = 0; i < kIn; ++i) x[i] = valid ? a.samples[i * a.stride + sidx] : 0.0f;
        // mode 0: nine higher-order targets; mode 1: tau (5) and S (5)
        const int t0 = net.mode == 1 ? kIn + kTargets : kIn;
        const int nt = net.mode == 1 ? kSgs : kTargets;
#pragma unroll
        for (int i = 0; i < kSgs; ++i) tg[i] = (valid && i < nt) ? a.samples[(t0 + i) * a.stride + sidx] : 0.0f;
        float v[32], z1[32];
#pragma unroll
        for (int i = 0; i < kIn; ++i) v[i] = valid ? (x[i] - net.mu[i]) * net.sinv[i] : 0.0f;
#pragma unroll
        for (int i = kIn; i < 32; ++i) v[i] = 0.0f;
        put_row32(sX, tid, v);
        if (GRAD) {
#pragma unroll
            for (int i = 0; i < 32; ++i) put_col(sBw, i, tid, v[i]);
            put_col(sBw, 64, tid, valid ? 1.0f : 0.0f);
        }
        tc_sync();
        if (tid == 0) mma_k32(tm, aX, aW1, &bar);
        ok = !__syncthreads_or(!tc::bar_wait(&bar, phase, a.spin_limit));
        phase ^= 1;
        if (!ok) break;
        tc::fence_after();
        tc::ld32(tc::lane_addr(tm, warp, 0), z1);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            z1[j] += net.b1[j];
            v[j] = gelu(z1[j]);
        }
        put_row32(sX, tid, v);
        if (GRAD) {
#pragma unroll
            for (int j = 0; j < 32; ++j) put_col(sBw, 32 + j, tid, v[j]);
        }
        tc_sync();
        if (tid == 0) mma_k32(tm, aX, aW2, &bar);
        ok = !__syncthreads_or(!tc::bar_wait(&bar, phase, a.spin_limit));
        phase ^= 1;
        if (!ok) break;
        tc::fence_after();
        tc::ld32(tc::lane_addr(tm, warp, 0), v);  // z2 - b2
        float z3 = net.b3;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            v[j] += net.b2[j];
            z3 += net.w3[j] * gelu(v[j]);
        }
        const float th = tanh_approx(z3);
        float dldth = 0.0f;  // d loss / d th
        if (net.mode == 1) {
            // tau_j + 2 nu_t S_j over the five deviatoric components
            float dnudth;
            const float nut = eddy_nu(net.nu, net.span, th, &dnudth) - net.nu;
            float dldnu = 0.0f;
#pragma unroll
            for (int i = 0; i < kSgs / 2; ++i) {
                const float r = tg[i] + 2.0f * nut * tg[kSgs / 2 + i];
                loss += valid ? a.wscale * r * r : 0.0f;
                dldnu += 4.0f * a.wscale * r * tg[kSgs / 2 + i];
            }
            dldth = dldnu * dnudth;
        } else {
            // t_j - (1 - s_h) p_j, s_h = 1 + span th, p_j the pre-collision moments
            const float oms = -net.span * th;
            float dlds = 0.0f;
#pragma unroll
            for (int i = 0; i < kTargets; ++i) {
                const float r = tg[i] - oms * x[10 + i];
                loss += valid ? a.wscale * r * r : 0.0f;
                dlds += 2.0f * a.wscale * r * x[10 + i];
            }
            dldth = dlds * net.span;
        }
        if (!GRAD) continue;
        const float d3 = valid ? dldth * (1.0f - th * th) : 0.0f;
        put_col(sAw, 64, tid, d3);
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const float h2 = gelu(v[j]);
            put_col(sBw, 80 + j, tid, h2);
            v[j] = d3 * net.w3[j] * gelu_grad(v[j]);  // delta2
            put_col(sAw, 32 + j, tid, v[j]);
        }
        put_row32(sX, tid, v);
        tc_sync();
        if (tid == 0) mma_k32(tm, aX, aW2T, &bar);  // dh1 = delta2 W2
        ok = !__syncthreads_or(!tc::bar_wait(&bar, phase, a.spin_limit));
        phase ^= 1;
        if (!ok) break;
        tc::fence_after();
        tc::ld32(tc::lane_addr(tm, warp, 0), v);
#pragma unroll
        for (int j = 0; j < 32; ++j) put_col(sAw, j, tid, v[j] * gelu_grad(z1[j]));  // delta1
        tc_sync();
        if (tid == 0) {
#pragma unroll
            for (int kk = 0; kk < 8; ++kk)
                tc::mma(tm + 32, tc::smem_desc(aAw + 256 * kk, 128, 2048), tc::smem_desc(aBw + 256 * kk, 128, 2048),
                        kIdescW, ntile > 0 || kk > 0);
            tc::commit(&bar);
        }
        ok = !__syncthreads_or(!tc::bar_wait(&bar, phase, a.spin_limit));
        phase ^= 1;
        if (!ok) break;
        tc::fence_after();
    }
    float* part = a.part + (long long)blockIdx.x * kPart;
    if (!ok) {
        if (tid == 0) atomicOr(a.status, kStatusWaitTimeout);
        tc::bar_wait(&bar, phase ^ 1, a.spin_limit);
    }
    // loss: block sum in a fixed order
    red[tid] = loss;
    __syncthreads();
    if (tid == 0) {
        float s = 0.0f;
        for (int i = 0; i < 128; ++i) s += red[i];
        part[kTrainable] = s;
    }
    if (GRAD) {
        tc::fence_after();
        float d[32];
        if (warp < 3) {
            const bool have = ok && ntile > 0;
            // lanes 0-31: dW1 rows, lanes 32-63: dW2 rows, lane 64: dW3 (row 64 of D)
            const int col = warp == 0 ? 32 : (warp == 1 ? 64 : 112);
            tc::ld32(tc::lane_addr(tm, warp, col), d);
            float db[32];
            tc::ld32(tc::lane_addr(tm, warp, 96), db);
            const int o = tid & 31;
            if (warp == 0) {
                for (int n = 0; n < 32; ++n) part[kW1 - kW1 + o * 32 + n] = have ? d[n] : 0.0f;
                part[kB1 - kW1 + o] = have ? db[0] : 0.0f;
            } else if (warp == 1) {
                for (int n = 0; n < 32; ++n) part[kW2 - kW1 + o * 32 + n] = have ? d[n] : 0.0f;
                part[kB2 - kW1 + o] = have ? db[0] : 0.0f;
            } else if (o == 0) {
                for (int n = 0; n < 32; ++n) part[kW3 - kW1 + n] = have ? d[n] : 0.0f;
                part[kB3 - kW1] = have ? db[0] : 0.0f;
            }
        }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) tc::dealloc(tm, 256);
}

// Gradient of the mean loss and the loss sum: fixed-order sums of the block partials.
__global__ void k_closure_reduce(const float* __restrict__ part, int blocks, float inv_batch,
                                 float* __restrict__ grad, double* __restrict__ loss) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > kTrainable) return;
    if (j == kTrainable) {
        double s = 0.0;
        for (int b = 0; b < blocks; ++b) s += part[(long long)b * kPart + j];
        *loss = s;
        return;
    }
    float s = 0.0f;
    for (int b = 0; b < blocks; ++b) s += part[(long long)b * kPart + j];
    grad[j] = s * inv_batch;
}

// Adam (Kingma and Ba) on the trainable block of the parameters, step t (from 1).
__global__ void k_closure_adam(float* __restrict__ p, const float* __restrict__ grad, float* __restrict__ m1,
                               float* __restrict__ m2, float lr, float b1, float b2, float eps, int t) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= kTrainable) return;
    const int in = (j < 1024) ? (j & 31) : 0;
    if (j < 1024 && in >= kIn) return;  // padded inputs of W1 stay zero
    const float g = grad[j];
    const float a = b1 * m1[j] + (1.0f - b1) * g;
    const float b = b2 * m2[j] + (1.0f - b2) * g * g;
    m1[j] = a;
    m2[j] = b;
    const float ah = a / (1.0f - powf(b1, (float)t)), bh = b / (1.0f - powf(b2, (float)t));
    p[kW1 + j] -= lr * ah / (sqrtf(bh) + eps);
}

int closure_train_smem() { return kTrSmem; }
int closure_part_floats() { return kPart; }

void launch_closure_train(const TrainArgs& a, bool grad, int grid, cudaStream_t st) {
    if (grad) {
        cudaFuncSetAttribute(k_closure_train<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrSmem);
        k_closure_train<true><<<grid, 128, kTrSmem, st>>>(a);
    } else {
        cudaFuncSetAttribute(k_closure_train<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrSmem);
        k_closure_train<false><<<grid, 128, kTrSmem, st>>>(a);
    }
}

void launch_closure_reduce(const float* part, int blocks, float inv_batch, float* grad, double* loss,
                           cudaStream_t st) {
    k_closure_reduce<<<(kTrainable + 1 + 255) / 256, 256, 0, st>>>(part, blocks, inv_batch, grad, loss);
}

void launch_closure_adam(float* params, const float* grad, float* m1, float* m2, float lr, float b1,
                         float b2, float eps, int t, cudaStream_t st) {
    k_closure_adam<<<(kTrainable + 255) / 256, 256, 0, st>>>(params, grad, m1, m2, lr, b1, b2, eps, t);
}

// ------------------------------------------------------------------ self tests
// D (128 x n) = A (128 x k) * B^T (n x k) through one MMA chain (k = 32 or 128, n = 32 or
// 112), operands rounded to bf16: checks the operand layout, the descriptors and the
// accumulator lanes against a host product.
__global__ void __launch_bounds__(128) k_tc_selftest(const float* __restrict__ A, const float* __restrict__ B,
                                                     float* __restrict__ D, int kdim, int n,
                                                     unsigned int* status, int spin) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tbase;
    unsigned char* sa = smem;
    unsigned char* sb = smem + 128 * kdim * 2;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int k = 0; k < kdim; ++k)
        *reinterpret_cast<uint16_t*>(sa + tc::kmajor_offset(tid, k, kdim)) = bf16_bits(A[tid * kdim + k]);
    if (tid < n)
        for (int k = 0; k < kdim; ++k)
            *reinterpret_cast<uint16_t*>(sb + tc::kmajor_offset(tid, k, kdim)) = bf16_bits(B[tid * kdim + k]);
    if (warp == 0) tc::alloc(&tbase, 128);
    if (tid == 0) tc::bar_init(&bar, 1);
    tc_sync();
    const uint32_t tm = tbase;
    const uint32_t sbo = (uint32_t)(kdim / 8) * 128;
    if (tid == 0) {
        const uint32_t id = tc::idesc_bf16(128, n);
        for (int kk = 0; kk < kdim / 16; ++kk)
            tc::mma(tm, tc::smem_desc(tc::smem_addr(sa) + 256 * kk, 128, sbo),
                    tc::smem_desc(tc::smem_addr(sb) + 256 * kk, 128, sbo), id, kk > 0);
        tc::commit(&bar);
    }
    const bool ok = !__syncthreads_or(!tc::bar_wait(&bar, 0, spin));
    if (!ok) {
        if (tid == 0) atomicOr(status, kStatusWaitTimeout);
        tc::bar_wait(&bar, 0, spin);
    } else {
        tc::fence_after();
        for (int c0 = 0; c0 < n; c0 += 32) {
            float v[32];
            tc::ld32(tc::lane_addr(tm, warp, c0), v);
            for (int j = 0; j < 32 && c0 + j < n; ++j) D[tid * n + c0 + j] = v[j];
        }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) tc::dealloc(tm, 128);
}

void launch_tc_selftest(const float* A, const float* B, float* D, int kdim, int n, unsigned int* status,
                        int spin, cudaStream_t st) {
    const int smem = 128 * kdim * 2 + 128 * kdim * 2;
    cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_tc_selftest<<<1, 128, smem, st>>>(A, B, D, kdim, n, status, spin);
}

}  // namespace clbm
