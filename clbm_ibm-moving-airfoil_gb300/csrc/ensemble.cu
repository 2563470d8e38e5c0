// ensemble.cu -- batched kernels that step many independent lattices at once.
//
// Each lattice of an ensemble keeps its own buffers; a device array of descriptors
// (EnsDesc) tells the batched kernels where they are. The marker, interpolation and
// force-sum kernels index the instance with blockIdx.y (each instance uses as many x-blocks
// as it needs, the rest leave); band-prepare and the box pass run one thread per force-box
// cell over a flat list of all instances' boxes. The bulk stream-collide pass runs over
// one flat list of tiles of all instances (runs of consecutive cells, or row segments for
// the two-cell 16-bit body), or with one row per block over groups of instances of equal
// row width, so lattices of different sizes share the GPU without tail effects; the tile
// width, the row mode and the number of persistent blocks are picked by timing at
// creation.
// Every per-cell and per-marker computation is the single-lattice code (lbm_device.cuh,
// ibm_device.cuh), so an instance gives the same bits as when it is stepped alone.
#include <algorithm>

#include "ibm_device.cuh"
#include "lbm_device.cuh"

namespace clbm {

__global__ void __launch_bounds__(kEnsMarkerBlock) kb_markers(const EnsDesc* __restrict__ d) {
    const EnsDesc& D = d[blockIdx.y];
    if (!D.has_ibm || (int)blockIdx.x * kEnsMarkerBlock >= D.a.n) return;  // whole block
    ibm_markers_body<true, kEnsMarkerBlock>(D.a, D.g, MotionF{}, D.m, blockIdx.x);
}

__global__ void __launch_bounds__(kSpreadBlock) kb_interp_spread(const EnsDesc* __restrict__ d) {
    const EnsDesc& D = d[blockIdx.y];
    const int m0 = ((blockIdx.x * kSpreadBlock + threadIdx.x) >> 5) * kSpreadMarkersPerWarp;
    if (!D.has_ibm || m0 >= D.a.n) return;  // whole warp
    ibm_interp_spread_body<kSpreadMarkersPerWarp>(D.a, D.g, m0, threadIdx.x & 31);
}

__global__ void __launch_bounds__(kTiledBlock) kb_interp_spread_tiled(const EnsDesc* __restrict__ d) {
    const EnsDesc& D = d[blockIdx.y];
    if (!D.has_ibm || (int)blockIdx.x * kTileMarkers >= D.a.n) return;  // whole block
    ibm_interp_spread_tiled_body(D.a, D.g, blockIdx.x);
}

__global__ void __launch_bounds__(kBoxBlock) kb_finish(const EnsDesc* __restrict__ d) {
    const EnsDesc& D = d[blockIdx.y];
    if (!D.has_ibm) return;
    ibm_finish_body<kBoxBlock>(D.a, D.g, blockIdx.x, gridDim.x);
}

// Force boxes of all members as one flat list: off_new[i] (off_old[i]) is the first flat
// index of member i's box of this compute_force call (of the previous call), i <= n, so the
// band-prepare and box passes run one thread per box cell over every member without
// blocks for members with small boxes. One block; n <= kEnsMaxMembers.
constexpr int kEnsMaxMembers = 4096;

__global__ void __launch_bounds__(1024) kb_box_scan(const EnsDesc* __restrict__ d, int n,
                                                    long long* __restrict__ off_new,
                                                    long long* __restrict__ off_old) {
    __shared__ int cn[kEnsMaxMembers], co[kEnsMaxMembers];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const EnsDesc& D = d[i];
        int a = 0, b = 0;
        if (D.has_ibm) {
            const long long s = D.a.dev->step + 1;
            const Band nb = load_band(D.a.dev, (int)(s & 1));
            const Band ob = load_band(D.a.dev, (int)((s - 1) & 1));
            a = nb.ilen * nb.jlen * nb.klen;
            b = ob.ilen * ob.jlen * ob.klen;
        }
        cn[i] = a;
        co[i] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long sa = 0, sb = 0;
        for (int i = 0; i < n; ++i) {
            off_new[i] = sa;
            off_old[i] = sb;
            sa += cn[i];
            sb += co[i];
        }
        off_new[n] = sa;
        off_old[n] = sb;
    }
}

// Member of flat index t: the last i with off[i] <= t.
__device__ __forceinline__ int member_of(const long long* __restrict__ off, int n, long long t) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(off + mid) <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int S, bool PULL>
__global__ void __launch_bounds__(kBoxBlock) kb_band_prepare_flat(const EnsDesc* __restrict__ d, int n,
                                                            const long long* __restrict__ off_new,
                                                            const long long* __restrict__ off_old,
                                                            int parity, bool compute_macro) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total_old = off_old[n];
    for (long long t = t0; t < total_old; t += stride) {
        const int i = member_of(off_old, n, t);
        const EnsDesc& D = d[i];
        const long long s = D.a.dev->step + 1;
        const Band ob = load_band(D.a.dev, (int)((s - 1) & 1));
        band_zero_cell(D.g, D.a.fx, D.a.fy, ob, (int)(t - off_old[i]));
    }
    if (!compute_macro) return;
    const long long total_new = off_new[n];
    for (long long t = t0; t < total_new; t += stride) {
        const int i = member_of(off_new, n, t);
        const EnsDesc& D = d[i];
        const long long s = D.a.dev->step + 1;
        const Band nb = load_band(D.a.dev, (int)(s & 1));
        band_macro_cell<S, PULL>((const typename Pop<S>::T*)D.f[parity], D.g, D.c, D.rho, D.ux, D.uy,
                                 D.uz, nb, (int)(t - off_new[i]));
    }
}

template <int S, bool PULL>
__global__ void __launch_bounds__(kBoxBlock) kb_box_flat(const EnsDesc* __restrict__ d, int n,
                                                   const long long* __restrict__ off_new, int parity) {
    using T = typename Pop<S>::T;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long total = off_new[n];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += stride) {
        const int i = member_of(off_new, n, t);
        const EnsDesc& D = d[i];
        ForceArgs fa{};
        fa.qx = D.a.fx;
        fa.qy = D.a.fy;
        fa.dev = D.a.dev;
        const Band b = load_band(D.a.dev, (int)(D.a.dev->cur & 1));
        box_pass_cell<S, PULL>((const T*)D.f[parity], (T*)D.f[parity ^ 1], D.g, D.c, fa, b,
                               (int)(t - off_new[i]));
    }
}

// Bulk pass over the flat tile list: tile t of instance i is tile (t - tile0[i]) of that
// instance, W cells each. Float32 (one cell per thread) takes runs of W consecutive cells in
// x-fastest order across row ends, so no lane idles at the end of a row; the 16-bit forms
// (two neighbouring cells of one row per thread) take segments of W cells of one row, so a
// warp's rows and their neighbour rows are the same for all its lanes. Each thread runs the
// single-lattice bodies (stream_collide_cell; pair_body: half2 loads, warp-shuffle x
// shifts), so an instance gives the same bits as when it is stepped alone.
template <int S, bool PULL, int W>
__global__ void __launch_bounds__(S == CLBM_STORE_F32 ? W : W / 2, S == CLBM_STORE_F32 ? 1024 / W : 2048 / W)
kb_bulk(const EnsDesc* __restrict__ d, const long long* __restrict__ tile0, int n, long long ntiles,
        int parity) {
    using T = typename Pop<S>::T;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        // instance of tile t: the last i with tile0[i] <= t
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(tile0 + mid) <= t) lo = mid;
            else hi = mid - 1;
        }
        const EnsDesc& D = d[lo];
        const Grid g = D.g;
        const Coef c = D.c;
        const unsigned local = (unsigned)(t - D.tile0);
        const T* fin = (const T*)D.f[parity];
        T* fout = (T*)D.f[parity ^ 1];
        ForceArgs fa{};
        if (D.has_ibm) {
            fa.dev = D.a.dev;
            fa.slot = (int)(D.a.dev->cur & 1);
        }
        if constexpr (S == CLBM_STORE_F32) {
            const unsigned i = local * W + threadIdx.x;
            if (i < (unsigned)D.cells) {
                const unsigned row = i / (unsigned)g.nx;
                const int x = (int)(i - row * (unsigned)g.nx);
                const int y = (int)(row % (unsigned)g.ny), z = (int)(row / (unsigned)g.ny);
                if (D.has_ibm) stream_collide_cell<S, PULL, kForceSkipBand>(fin, fout, g, c, fa, x, y, z);
                else stream_collide_cell<S, PULL, kForceNone>(fin, fout, g, c, fa, x, y, z);
            }
        } else {
            const int nseg = (g.nx + W - 1) / W;
            const int r = (int)local / nseg;   // row z * ny + y
            const int x0 = ((int)local - r * nseg) * W + 2 * threadIdx.x;
            const int y = r % g.ny, z = r / g.ny;
            if (D.has_ibm) pair_body<S, PULL, kForceSkipBand>(fin, fout, g, c, fa, x0, y, z);
            else pair_body<S, PULL, kForceNone>(fin, fout, g, c, fa, x0, y, z);
        }
    }
}

// 16-bit forms, whole rows per block: tile t of a group is rows R (t - tile0[i]) ...
// R (t - tile0[i]) + R - 1 of instance i (row index z * ny + y, y fastest), computed one
// after the other; the block's warps cover a row with two cells per thread (blockDim.x >=
// Nx / 2, the smallest multiple of 32). Instances are grouped by that width, one launch
// per group, so a 150-, 200- or 300-cell row costs 3, 4 or 5 warps and the row (y, z)
// stays uniform across the block. The instance lookup and its descriptor reads (dependent
// loads) are paid once per R rows.
template <int S, bool PULL, bool IDX32>
__global__ void __launch_bounds__(256, 4) kb_bulk_row(const EnsDesc* __restrict__ d,
                                                    const long long* __restrict__ tile0, int n,
                                                    long long ntiles, int parity, int R) {
    using T = typename Pop<S>::T;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(tile0 + mid) <= t) lo = mid;
            else hi = mid - 1;
        }
        const EnsDesc& D = d[lo];
        const Grid g = D.g;
        const Coef c = D.c;
        const int rows = g.ny * g.nz;
        const int r0 = (int)(t - D.tile0) * R;
        const int r1 = min(r0 + R, rows);
        const T* fin = (const T*)D.f[parity];
        T* fout = (T*)D.f[parity ^ 1];
        ForceArgs fa{};
        if (D.has_ibm) {
            fa.dev = D.a.dev;
            fa.slot = (int)(D.a.dev->cur & 1);
            for (int r = r0; r < r1; ++r)
                pair_body<S, PULL, kForceSkipBand, IDX32>(fin, fout, g, c, fa, 2 * threadIdx.x, r % g.ny, r / g.ny);
        } else {
            for (int r = r0; r < r1; ++r)
                pair_body<S, PULL, kForceNone, IDX32>(fin, fout, g, c, fa, 2 * threadIdx.x, r % g.ny, r / g.ny);
        }
    }
}

// Float32, whole rows per block (R per tile, as above): one cell per thread, blockDim.x >=
// Nx (a multiple of 32).
template <bool PULL>
__global__ void __launch_bounds__(512) kb_bulk_row_f32(const EnsDesc* __restrict__ d,
                                                       const long long* __restrict__ tile0, int n,
                                                       long long ntiles, int parity, int R) {
    using T = typename Pop<CLBM_STORE_F32>::T;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(tile0 + mid) <= t) lo = mid;
            else hi = mid - 1;
        }
        const EnsDesc& D = d[lo];
        const Grid g = D.g;
        const Coef c = D.c;
        const int x = threadIdx.x;
        if (x >= g.nx) continue;
        const int rows = g.ny * g.nz;
        const int r0 = (int)(t - D.tile0) * R;
        const int r1 = min(r0 + R, rows);
        const T* fin = (const T*)D.f[parity];
        T* fout = (T*)D.f[parity ^ 1];
        ForceArgs fa{};
        if (D.has_ibm) {
            fa.dev = D.a.dev;
            fa.slot = (int)(D.a.dev->cur & 1);
            for (int r = r0; r < r1; ++r)
                stream_collide_cell<CLBM_STORE_F32, PULL, kForceSkipBand>(fin, fout, g, c, fa, x, r % g.ny, r / g.ny);
        } else {
            for (int r = r0; r < r1; ++r)
                stream_collide_cell<CLBM_STORE_F32, PULL, kForceNone>(fin, fout, g, c, fa, x, r % g.ny, r / g.ny);
        }
    }
}

void launch_ens_bulk_rows(int storage, bool pull, int threads, int rows_per_tile, bool idx32,
                          const EnsDesc* d, const long long* tile0, int n, long long ntiles,
                          int parity, int grid, cudaStream_t st) {
    const int R = rows_per_tile;
    if (storage == CLBM_STORE_F32) {
        if (pull) kb_bulk_row_f32<true><<<grid, threads, 0, st>>>(d, tile0, n, ntiles, parity, R);
        else kb_bulk_row_f32<false><<<grid, threads, 0, st>>>(d, tile0, n, ntiles, parity, R);
        return;
    }
#define CLBM_ENS_ROW(S_)                                                                                  \
    {                                                                                                     \
        if (pull && idx32) kb_bulk_row<S_, true, true><<<grid, threads, 0, st>>>(d, tile0, n, ntiles, parity, R);  \
        else if (pull) kb_bulk_row<S_, true, false><<<grid, threads, 0, st>>>(d, tile0, n, ntiles, parity, R);     \
        else if (idx32) kb_bulk_row<S_, false, true><<<grid, threads, 0, st>>>(d, tile0, n, ntiles, parity, R);    \
        else kb_bulk_row<S_, false, false><<<grid, threads, 0, st>>>(d, tile0, n, ntiles, parity, R);             \
    }
    if (storage == CLBM_STORE_F16S) CLBM_ENS_ROW(CLBM_STORE_F16S)
    else if (storage == CLBM_STORE_BF16S) CLBM_ENS_ROW(CLBM_STORE_BF16S)
#undef CLBM_ENS_ROW
}

// ---------------------------------------------------------------- one persistent launch
// The whole ensemble step as one cooperative launch (every block resident at once), the
// form that one CUDA graph node replays: the IBM chain's dependent phases are separated by
// a grid barrier, and the bulk pass's tiles are shared out over the phases, so that every
// block does its part of the latency-bound chain and then bulk tiles until the next
// barrier:
//   1 markers of all members (the last virtual block of a member writes its force band)
//   2 flat offsets of all force boxes (warp 0 of block 0)           + bulk tiles
//   3 band prepare over the flat box-cell list                     + bulk tiles
//   4 interpolation and spreading, two markers per warp            + bulk tiles
//   5 force sums (virtual blocks per member) and the box pass (16-bit: by box rows, a
//     64-cell segment per warp)                                     + the remaining bulk tiles
// A warp's bulk tile is a 64-cell row segment (16-bit forms: the two-cell body, x shifts
// by warp shuffles) or a run of 32 consecutive cells across row ends (float32); a block
// takes kPersTileWarps consecutive warp tiles of one member at a time, whose constants it
// reads from the kernel's parameter table (EnsPersTable). Every per-cell and per-marker
// computation is the body the separate launches use; data written earlier in the launch
// (bands, offsets, macro fields, marker positions and forces, force fields) is read with
// plain or L2 loads after a barrier, never through the read-only path (the populations
// read are those of the previous step).
constexpr int kPersThreads = 256;
constexpr int kPersWarps = kPersThreads / 32;
constexpr int kBarrierPolls = 1 << 20;   // with 32 ns sleeps and an L2 round trip per poll: under a second

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acq_rel_u32(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// Barrier of the blocks of a cooperative launch: bar[0] arrivals, bar[1] generation,
// bar[2] error bits. `expect` blocks must arrive (gridDim.x; a larger value is the
// timeout self-test). A block waits at most kBarrierPolls polls; then it sets bar[2] and
// goes on (the step's results are invalid and the host reports the error).
__device__ __forceinline__ void grid_barrier(unsigned* bar, unsigned expect) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = ld_acquire_u32(bar + 1);
        __threadfence();
        const unsigned arrived = atom_add_acq_rel_u32(bar, 1u) + 1u;
        if (arrived == expect) {
            bar[0] = 0u;                       // ordered before the release below
            st_release_u32(bar + 1, gen + 1u);
        } else {
            bool ok = false;
            for (int it = 0; it < kBarrierPolls; ++it) {
                if (ld_acquire_u32(bar + 1) != gen) { ok = true; break; }
                __nanosleep(32);
            }
            if (!ok) atomicOr(bar + 2, 1u);
        }
        __threadfence();
    }
    __syncthreads();
}

// Phase clock of the persistent step: thread 0 of block 0 records the global timer (ns)
// at the start and after each barrier into p.stamps[0..5] (when p.stamps is set).
__device__ __forceinline__ void pers_stamp(const EnsPersArgs& p, int k) {
    if (p.stamps && blockIdx.x == 0 && threadIdx.x == 0) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        p.stamps[k] = t;
    }
}

// Member of flat index t over offsets written earlier in this launch (L2 loads).
__device__ __forceinline__ int member_of_cg(const long long* off, int n, long long t) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldcg(off + mid) <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Block tiles [b0, b1) of the bulk pass: a block tile is kPersTileWarps consecutive warp
// tiles of one member, so the member number is the same in the whole block and its
// constants come from the parameter table (constant bank) like a separate launch's.
template <int S, bool PULL, bool IDX32>
__device__ __forceinline__ void pers_bulk(const EnsPersTable& tb, const EnsPersArgs& p, int b0, int b1) {
    using T = typename Pop<S>::T;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int bt = b0 + (int)blockIdx.x; bt < b1; bt += (int)gridDim.x) {
        int lo = 0, hi = p.n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tb.bt0[mid] <= bt) lo = mid;
            else hi = mid - 1;
        }
        const EnsMember& M = tb.m[lo];
        const int w = (bt - tb.bt0[lo]) * kPersTileWarps + warp;   // warp tile of member lo
        if (w >= M.wtiles) continue;                                // warp-uniform
        const T* fin = (const T*)M.f[p.parity];
        T* fout = (T*)M.f[p.parity ^ 1];
        ForceArgs fa{};
        fa.dev = M.dev;
        fa.slot = (int)(M.dev->cur & 1);
        if constexpr (S == CLBM_STORE_F32) {
            const unsigned k = (unsigned)w * 32u + (unsigned)lane;
            if (k < (unsigned)M.cells) {
                const unsigned row = k / (unsigned)M.g.nx;
                const int x = (int)(k - row * (unsigned)M.g.nx);
                const int y = (int)(row % (unsigned)M.g.ny), z = (int)(row / (unsigned)M.g.ny);
                stream_collide_cell<S, PULL, kForceSkipBand, IDX32>(fin, fout, M.g, M.c, fa, x, y, z);
            }
        } else {
            const unsigned nseg = (unsigned)(M.g.nx + 63) / 64u;
            const unsigned r = (unsigned)w / nseg;   // row z * ny + y
            const int x0 = (int)((unsigned)w - r * nseg) * 64 + 2 * lane;
            const int y = (int)(r % (unsigned)M.g.ny), z = (int)(r / (unsigned)M.g.ny);
            pair_body<S, PULL, kForceSkipBand, IDX32>(fin, fout, M.g, M.c, fa, x0, y, z);
        }
    }
}

template <int S, bool PULL, bool IDX32>
__global__ void __launch_bounds__(kPersThreads, S == CLBM_STORE_F32 ? 2 : 3)
kb_step_persistent(const EnsDesc* __restrict__ d, EnsPersArgs p, EnsPersTable tb) {
    using T = typename Pop<S>::T;
    const int n = p.n;
    const unsigned nb = gridDim.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long gthread = (long long)blockIdx.x * kPersThreads + threadIdx.x;
    const long long nthread = (long long)gridDim.x * kPersThreads;
    pers_stamp(p, 0);
    // 1: markers, virtual blocks of kEnsMarkerBlock markers (block-uniform branches)
    for (long long v = blockIdx.x; v < p.mk_total; v += nb) {
        const int i = member_of(p.mk0, n, v);
        const EnsDesc& D = d[i];
        ibm_markers_body<true, kEnsMarkerBlock>(D.a, D.g, MotionF{}, D.m, (int)(v - __ldg(p.mk0 + i)));
    }
    grid_barrier(p.bar, nb);
    pers_stamp(p, 1);
    // 2: flat offsets of this call's and the previous call's boxes
    if (blockIdx.x == 0 && warp == 0) {
        long long sa = 0, sb = 0, sr = 0;
        for (int base = 0; base < n; base += 32) {
            const int i = base + lane;
            long long a = 0, b = 0, rw = 0;
            if (i < n && d[i].has_ibm) {
                const IbmDev* dev = d[i].a.dev;
                const long long s = dev->step + 1;
                const Band nbd = load_band(dev, (int)(s & 1));
                const Band obd = load_band(dev, (int)((s - 1) & 1));
                a = (long long)nbd.ilen * nbd.jlen * nbd.klen;
                b = (long long)obd.ilen * obd.jlen * obd.klen;
                // box pass by rows: 64-cell segments from i0 rounded down to even
                if (nbd.ilen > 0)
                    rw = (long long)((nbd.i0 + nbd.ilen - (nbd.i0 & ~1) + 63) / 64) * nbd.jlen * nbd.klen;
            }
            long long ia = a, ib = b, ir = rw;   // inclusive warp scans
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long ua = __shfl_up_sync(0xffffffffu, ia, o);
                const long long ub = __shfl_up_sync(0xffffffffu, ib, o);
                const long long ur = __shfl_up_sync(0xffffffffu, ir, o);
                if (lane >= o) { ia += ua; ib += ub; ir += ur; }
            }
            if (i < n) {
                p.off_new[i] = sa + ia - a;
                p.off_old[i] = sb + ib - b;
                p.off_rows[i] = sr + ir - rw;
            }
            sa += __shfl_sync(0xffffffffu, ia, 31);
            sb += __shfl_sync(0xffffffffu, ib, 31);
            sr += __shfl_sync(0xffffffffu, ir, 31);
        }
        if (lane == 0) {
            p.off_new[n] = sa;
            p.off_old[n] = sb;
            p.off_rows[n] = sr;
        }
    }
    pers_bulk<S, PULL, IDX32>(tb, p, p.bt_split[0], p.bt_split[1]);
    grid_barrier(p.bar, nb);
    pers_stamp(p, 2);
    // 3: band prepare over the flat list (zero the previous box, macro on the new one)
    {
        const long long total_old = __ldcg(p.off_old + n);
        for (long long t = gthread; t < total_old; t += nthread) {
            const int i = member_of_cg(p.off_old, n, t);
            const EnsDesc& D = d[i];
            const long long s = D.a.dev->step + 1;
            const Band ob = load_band(D.a.dev, (int)((s - 1) & 1));
            band_zero_cell(D.g, D.a.fx, D.a.fy, ob, (int)(t - __ldcg(p.off_old + i)));
        }
        if (p.compute_macro) {
            const long long total_new = __ldcg(p.off_new + n);
            for (long long t = gthread; t < total_new; t += nthread) {
                const int i = member_of_cg(p.off_new, n, t);
                const EnsDesc& D = d[i];
                const long long s = D.a.dev->step + 1;
                const Band nbd = load_band(D.a.dev, (int)(s & 1));
                band_macro_cell<S, PULL>((const T*)D.f[p.parity], D.g, D.c, D.rho, D.ux, D.uy, D.uz,
                                         nbd, (int)(t - __ldcg(p.off_new + i)));
            }
        }
    }
    pers_bulk<S, PULL, IDX32>(tb, p, p.bt_split[1], p.bt_split[2]);
    grid_barrier(p.bar, nb);
    pers_stamp(p, 3);
    // 4: interpolation and spreading, kSpreadMarkersPerWarp markers per warp
    {
        const long long gw = (long long)blockIdx.x * kPersWarps + warp;
        for (long long w = gw; w < p.sw_total; w += (long long)nb * kPersWarps) {
            const int i = member_of(p.sw0, n, w);
            const EnsDesc& D = d[i];
            ibm_interp_spread_body<kSpreadMarkersPerWarp>(
                D.a, D.g, (int)(w - __ldg(p.sw0 + i)) * kSpreadMarkersPerWarp, lane);
        }
    }
    pers_bulk<S, PULL, IDX32>(tb, p, p.bt_split[2], p.bt_split[3]);
    grid_barrier(p.bar, nb);
    pers_stamp(p, 4);
    // 5: force sums (virtual blocks of kPersThreads threads per member) and the box pass
    for (long long v = blockIdx.x; v < (long long)n * p.fin_blocks; v += nb) {
        const int i = (int)(v / p.fin_blocks);
        const EnsDesc& D = d[i];
        if (D.has_ibm) ibm_finish_body<kPersThreads>(D.a, D.g, (int)(v % p.fin_blocks), p.fin_blocks);
    }
    if constexpr (S == CLBM_STORE_F32) {
        // one box cell per thread (the flat box pass of the separate launches)
        const long long total = __ldcg(p.off_new + n);
        for (long long t = gthread; t < total; t += nthread) {
            const int i = member_of_cg(p.off_new, n, t);
            const EnsDesc& D = d[i];
            ForceArgs fa{};
            fa.qx = D.a.fx;
            fa.qy = D.a.fy;
            fa.dev = D.a.dev;
            const Band b = load_band(D.a.dev, (int)(D.a.dev->cur & 1));
            box_pass_cell<S, PULL>((const T*)D.f[p.parity], (T*)D.f[p.parity ^ 1], D.g, D.c, fa, b,
                                   (int)(t - __ldcg(p.off_new + i)));
        }
    } else {
        // by rows of the box, a 64-cell segment per warp with the two-cell body (the single
        // lattice's box pass; the same bits as one cell per thread)
        const long long total = __ldcg(p.off_rows + n);
        for (long long w = (long long)blockIdx.x * kPersWarps + warp; w < total; w += (long long)nb * kPersWarps) {
            const int i = member_of_cg(p.off_rows, n, w);
            const EnsDesc& D = d[i];
            ForceArgs fa{};
            fa.qx = D.a.fx;
            fa.qy = D.a.fy;
            fa.dev = D.a.dev;
            fa.slot = (int)(D.a.dev->cur & 1);
            const Band b = load_band(D.a.dev, fa.slot);
            const int xa = b.i0 & ~1;
            const int nseg = (b.i0 + b.ilen - xa + 63) / 64;
            const int local = (int)(w - __ldcg(p.off_rows + i));
            const int seg = local % nseg, r = local / nseg;
            const int y = pmod(b.j0 + r % b.jlen, D.g.ny), z = pmod(b.k0 + r / b.jlen, D.g.nz);
            pair_body<S, PULL, kForceOnlyBand, IDX32>((const T*)D.f[p.parity], (T*)D.f[p.parity ^ 1], D.g,
                                                      D.c, fa, xa + seg * 64 + 2 * lane, y, z);
        }
    }
    pers_bulk<S, PULL, IDX32>(tb, p, p.bt_split[3], p.bt_split[4]);
    pers_stamp(p, 5);
}

// Self-test of the bounded barrier: every block waits for one block more than the launch
// has, so each wait runs out and sets the error bit.
__global__ void __launch_bounds__(kPersThreads) kb_barrier_selftest(unsigned* bar) {
    grid_barrier(bar, gridDim.x + 1);
}

template <int S, bool PULL, bool IDX32>
static int pers_occupancy() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kb_step_persistent<S, PULL, IDX32>, kPersThreads, 0) != cudaSuccess)
        return 0;
    return nb;
}

template <int S, bool PULL, bool IDX32>
static cudaError_t pers_launch(const EnsDesc* d, const EnsPersArgs& p, const EnsPersTable& t, int grid,
                               cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kPersThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kb_step_persistent<S, PULL, IDX32>, d, p, t);
}

int ens_persistent_blocks_per_sm(int storage, bool idx32) {
    int a = 0, b = 0;
#define CLBM_PERS_OCC(S_)                                                              \
    if (idx32) { a = pers_occupancy<S_, true, true>(); b = pers_occupancy<S_, false, true>(); } \
    else { a = pers_occupancy<S_, true, false>(); b = pers_occupancy<S_, false, false>(); }
    if (storage == CLBM_STORE_F32) { CLBM_PERS_OCC(CLBM_STORE_F32) }
    else if (storage == CLBM_STORE_F16S) { CLBM_PERS_OCC(CLBM_STORE_F16S) }
    else { CLBM_PERS_OCC(CLBM_STORE_BF16S) }
#undef CLBM_PERS_OCC
    return std::min(a, b);
}

cudaError_t launch_ens_persistent(int storage, bool pull, bool idx32, const EnsDesc* d,
                                  const EnsPersArgs& p, const EnsPersTable& t, int grid,
                                  cudaStream_t st) {
#define CLBM_PERS_GO(S_)                                                                  \
    if (pull && idx32) return pers_launch<S_, true, true>(d, p, t, grid, st);            \
    if (pull) return pers_launch<S_, true, false>(d, p, t, grid, st);                    \
    if (idx32) return pers_launch<S_, false, true>(d, p, t, grid, st);                   \
    return pers_launch<S_, false, false>(d, p, t, grid, st);
    if (storage == CLBM_STORE_F32) { CLBM_PERS_GO(CLBM_STORE_F32) }
    else if (storage == CLBM_STORE_F16S) { CLBM_PERS_GO(CLBM_STORE_F16S) }
    else { CLBM_PERS_GO(CLBM_STORE_BF16S) }
#undef CLBM_PERS_GO
}

cudaError_t launch_ens_barrier_selftest(unsigned* bar, int grid, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kPersThreads);
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kb_barrier_selftest, bar);
}

#define CLBM_ENS_STORE(storage, ...)                                                         \
    switch (storage) {                                                                       \
        case CLBM_STORE_F32: { constexpr int S_ = CLBM_STORE_F32; __VA_ARGS__; } break;     \
        case CLBM_STORE_F16S: { constexpr int S_ = CLBM_STORE_F16S; __VA_ARGS__; } break;   \
        default: { constexpr int S_ = CLBM_STORE_BF16S; __VA_ARGS__; } break;               \
    }

void launch_ens_markers(const EnsDesc* d, int n, int blocks, cudaStream_t st) {
    if (blocks < 1) return;
    kb_markers<<<dim3(blocks, n), kEnsMarkerBlock, 0, st>>>(d);
}

void launch_ens_interp_spread(const EnsDesc* d, int n, int blocks, cudaStream_t st) {
    if (blocks < 1) return;
    if (spread_tiled()) {
        // a block of the direct form covers (kSpreadBlock / 32) * kSpreadMarkersPerWarp
        // markers; a tiled block kTileMarkers
        const int per = (kSpreadBlock / 32) * kSpreadMarkersPerWarp;
        kb_interp_spread_tiled<<<dim3((blocks * per + kTileMarkers - 1) / kTileMarkers, n), kTiledBlock, 0, st>>>(d);
        return;
    }
    kb_interp_spread<<<dim3(blocks, n), kSpreadBlock, 0, st>>>(d);
}

void launch_ens_finish(const EnsDesc* d, int n, cudaStream_t st) {
    // 64-thread blocks (they run beside the bulk pass, whose blocks free room for them one
    // at a time), kFinishBlocks per member: the same threads per member as 16 blocks of 256
    kb_finish<<<dim3(kFinishBlocks, n), kBoxBlock, 0, st>>>(d);
}

void launch_ens_box_scan(const EnsDesc* d, int n, long long* off_new, long long* off_old, cudaStream_t st) {
    kb_box_scan<<<1, 1024, 0, st>>>(d, n, off_new, off_old);
}

void launch_ens_band_prepare_flat(int storage, bool pull, const EnsDesc* d, int n, const long long* off_new,
                                  const long long* off_old, int parity, bool compute_macro, int grid,
                                  cudaStream_t st) {
    CLBM_ENS_STORE(storage, {
        if (pull) kb_band_prepare_flat<S_, true><<<grid, kBoxBlock, 0, st>>>(d, n, off_new, off_old, parity, compute_macro);
        else kb_band_prepare_flat<S_, false><<<grid, kBoxBlock, 0, st>>>(d, n, off_new, off_old, parity, compute_macro);
    });
}

void launch_ens_box_flat(int storage, bool pull, const EnsDesc* d, int n, const long long* off_new, int parity,
                         int grid, cudaStream_t st) {
    CLBM_ENS_STORE(storage, {
        if (pull) kb_box_flat<S_, true><<<grid, kBoxBlock, 0, st>>>(d, n, off_new, parity);
        else kb_box_flat<S_, false><<<grid, kBoxBlock, 0, st>>>(d, n, off_new, parity);
    });
}

template <int S, bool PULL>
static void ens_bulk(int bx, const EnsDesc* d, const long long* tile0, int n, long long ntiles,
                     int parity, int grid, cudaStream_t st) {
    constexpr int kDiv = S == CLBM_STORE_F32 ? 1 : 2;  // cells per thread
    if (bx == 256) kb_bulk<S, PULL, 256><<<grid, 256 / kDiv, 0, st>>>(d, tile0, n, ntiles, parity);
    else kb_bulk<S, PULL, 128><<<grid, 128 / kDiv, 0, st>>>(d, tile0, n, ntiles, parity);
}

void launch_ens_bulk(int storage, bool pull, int bx, const EnsDesc* d, const long long* tile0,
                     int n, long long ntiles, int parity, int grid, cudaStream_t st) {
    CLBM_ENS_STORE(storage, {
        if (pull) ens_bulk<S_, true>(bx, d, tile0, n, ntiles, parity, grid, st);
        else ens_bulk<S_, false>(bx, d, tile0, n, ntiles, parity, grid, st);
    });
}

}  // namespace clbm
