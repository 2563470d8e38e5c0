// ensemble.cu -- batched kernels that step many independent lattices at once.
//
// Each lattice of an ensemble keeps its own buffers; a device array of descriptors
// (EnsDesc) tells the batched kernels where they are. The IBM kernels index the instance
// with blockIdx.y (each instance uses as many x-blocks as it needs, the rest leave). The
// bulk stream-collide pass runs persistent blocks over one flat list of tiles (runs of
// consecutive cells) of all instances, so lattices of different sizes share the GPU without tail effects;
// the tile width and the number of persistent blocks are picked by timing at creation.
// Every per-cell and per-marker computation is the single-lattice code (lbm_device.cuh,
// ibm_device.cuh), so an instance gives the same bits as when it is stepped alone.
#include <algorithm>

#include "ibm_device.cuh"
#include "lbm_device.cuh"

namespace clbm {

__global__ void __launch_bounds__(kMarkerBlock) kb_markers(const EnsDesc* __restrict__ d) {
    const EnsDesc& D = d[blockIdx.y];
    if (!D.has_ibm || (int)blockIdx.x * kMarkerBlock >= D.a.n) return;  // whole block
    ibm_markers_body<true>(D.a, D.g, MotionF{}, D.m, blockIdx.x);
}

template <int S, bool PULL>
__global__ void __launch_bounds__(256) kb_band_prepare(const EnsDesc* __restrict__ d, int parity,
                                                       bool compute_macro) {
    const EnsDesc& D = d[blockIdx.y];
    if (!D.has_ibm) return;
    band_prepare_body<S, PULL>((const typename Pop<S>::T*)D.f[parity], D.g, D.c, D.a.dev, D.a.fx,
                               D.a.fy, D.rho, D.ux, D.uy, D.uz, compute_macro, blockIdx.x,
                               gridDim.x);
}

__global__ void __launch_bounds__(kSpreadBlock) kb_interp_spread(const EnsDesc* __restrict__ d) {
    const EnsDesc& D = d[blockIdx.y];
    const int m = (blockIdx.x * kSpreadBlock + threadIdx.x) >> 5;
    if (!D.has_ibm || m >= D.a.n) return;  // whole warp
    ibm_interp_spread_body(D.a, D.g, m, threadIdx.x & 31);
}

__global__ void __launch_bounds__(kFinishBlock) kb_finish(const EnsDesc* __restrict__ d) {
    const EnsDesc& D = d[blockIdx.y];
    if (!D.has_ibm) return;
    ibm_finish_body(D.a, D.g, blockIdx.x, gridDim.x);
}

template <int S, bool PULL>
__global__ void __launch_bounds__(256) kb_box(const EnsDesc* __restrict__ d, int parity) {
    const EnsDesc& D = d[blockIdx.y];
    if (!D.has_ibm) return;
    ForceArgs fa{};
    fa.qx = D.a.fx;
    fa.qy = D.a.fy;
    fa.dev = D.a.dev;
    using T = typename Pop<S>::T;
    box_pass_body<S, PULL>((const T*)D.f[parity], (T*)D.f[parity ^ 1], D.g, D.c, fa, blockIdx.x,
                           gridDim.x);
}

template <int S, bool PULL, int BX>
__global__ void __launch_bounds__(BX) kb_bulk(const EnsDesc* __restrict__ d,
                                              const long long* __restrict__ tile0, int n,
                                              long long ntiles, int parity) {
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
        // tiles run over the instance's cells in x-fastest order across row ends, so no
        // lane idles at the end of a row that is not a multiple of the tile width
        const unsigned i = (unsigned)(t - D.tile0) * BX + threadIdx.x;
        if (i >= (unsigned)D.cells) continue;
        const unsigned row = i / (unsigned)g.nx;
        const int x = (int)(i - row * (unsigned)g.nx);
        const int y = (int)(row % (unsigned)g.ny), z = (int)(row / (unsigned)g.ny);
        const T* fin = (const T*)D.f[parity];
        T* fout = (T*)D.f[parity ^ 1];
        if (D.has_ibm) {
            ForceArgs fa{};
            fa.qx = D.a.fx;
            fa.qy = D.a.fy;
            fa.dev = D.a.dev;
            stream_collide_cell<S, PULL, kForceSkipBand>(fin, fout, g, D.c, fa, x, y, z);
        } else {
            stream_collide_cell<S, PULL, kForceNone>(fin, fout, g, D.c, ForceArgs{}, x, y, z);
        }
    }
}

#define CLBM_ENS_STORE(storage, ...)                                                         \
    switch (storage) {                                                                       \
        case CLBM_STORE_F32: { constexpr int S_ = CLBM_STORE_F32; __VA_ARGS__; } break;     \
        case CLBM_STORE_F16S: { constexpr int S_ = CLBM_STORE_F16S; __VA_ARGS__; } break;   \
        default: { constexpr int S_ = CLBM_STORE_BF16S; __VA_ARGS__; } break;               \
    }

void launch_ens_markers(const EnsDesc* d, int n, int blocks, cudaStream_t st) {
    if (blocks < 1) return;
    kb_markers<<<dim3(blocks, n), kMarkerBlock, 0, st>>>(d);
}

void launch_ens_band_prepare(int storage, bool pull, const EnsDesc* d, int n, int parity,
                             bool compute_macro, int blocks, cudaStream_t st) {
    const dim3 grid(std::max(blocks, 1), n);
    CLBM_ENS_STORE(storage, {
        if (pull) kb_band_prepare<S_, true><<<grid, 256, 0, st>>>(d, parity, compute_macro);
        else kb_band_prepare<S_, false><<<grid, 256, 0, st>>>(d, parity, compute_macro);
    });
}

void launch_ens_interp_spread(const EnsDesc* d, int n, int blocks, cudaStream_t st) {
    if (blocks < 1) return;
    kb_interp_spread<<<dim3(blocks, n), kSpreadBlock, 0, st>>>(d);
}

void launch_ens_finish(const EnsDesc* d, int n, cudaStream_t st) {
    kb_finish<<<dim3(kFinishBlocks, n), kFinishBlock, 0, st>>>(d);
}

void launch_ens_box(int storage, bool pull, const EnsDesc* d, int n, int parity, int blocks,
                    cudaStream_t st) {
    const dim3 grid(std::max(blocks, 1), n);
    CLBM_ENS_STORE(storage, {
        if (pull) kb_box<S_, true><<<grid, 256, 0, st>>>(d, parity);
        else kb_box<S_, false><<<grid, 256, 0, st>>>(d, parity);
    });
}

template <int S, bool PULL>
static void ens_bulk(int bx, const EnsDesc* d, const long long* tile0, int n, long long ntiles,
                     int parity, int grid, cudaStream_t st) {
    if (bx == 256) kb_bulk<S, PULL, 256><<<grid, 256, 0, st>>>(d, tile0, n, ntiles, parity);
    else kb_bulk<S, PULL, 128><<<grid, 128, 0, st>>>(d, tile0, n, ntiles, parity);
}

void launch_ens_bulk(int storage, bool pull, int bx, const EnsDesc* d, const long long* tile0,
                     int n, long long ntiles, int parity, int grid, cudaStream_t st) {
    CLBM_ENS_STORE(storage, {
        if (pull) ens_bulk<S_, true>(bx, d, tile0, n, ntiles, parity, grid, st);
        else ens_bulk<S_, false>(bx, d, tile0, n, ntiles, parity, grid, st);
    });
}

}  // namespace clbm
