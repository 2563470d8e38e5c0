// noalloc.cu -- an entry point for callers that cannot allocate device memory.
//
// ibm_force_sums_noalloc computes the same double-precision force sums as the force-sum
// kernel of an IBM step (sum of the clipped Eulerian force over all cells and sum of the
// marker forces), but over force fields and marker forces that the caller already holds in
// device memory, for example fields produced by another solver component or exported into
// a framework tensor. Some callers cannot call cudaMalloc at this point: a real-time loop
// whose memory budget is fixed up front, or a host whose device memory is owned by a pool
// allocator it cannot reach (an allocation outside that pool would fail or fragment it).
// For them this entry point allocates nothing: its per-block partial sums live in a
// file-scope __device__ array of fixed size, which every GPU that loads this library holds
// until the process exits.
//
// The call is synchronous: it ends by copying the sums to host memory and waiting for
// `stream`. A stream that is being captured into a CUDA graph cannot do either, so a call
// on a capturing stream (or on the legacy default stream while another stream captures in
// global mode) is refused with CLBM_ERR_STATE before any work is issued, and the caller's
// capture stays valid.
#include <cstdio>
#include <mutex>

#include "clbm_internal.cuh"

namespace {

// Maximum number of reduction blocks, and cells each block covers: the largest lattice the
// entry point accepts is kNoAllocBlocks * kNoAllocCellsPerBlock = 67,108,864 cells.
constexpr int kNoAllocBlocks = 16384;
constexpr int kNoAllocCellsPerBlock = 4096;
constexpr int kNoAllocThreads = 256;
constexpr int kMaxDevices = 64;

// Scratch shared by every call on a device: partial sums [block][4], the last-block
// ticket and the final four sums. Host code must not pass these names to a kernel (on the
// host they are stand-ins, not device addresses); their device addresses come from
// cudaGetSymbolAddress below.
__device__ __align__(256) double g_noalloc_part[kNoAllocBlocks][4];
__device__ __align__(256) unsigned int g_noalloc_ticket;
__device__ __align__(256) double g_noalloc_out[4];

struct Scratch {
    double* part = nullptr;
    unsigned int* ticket = nullptr;
    double* out = nullptr;
};
Scratch g_scratch[kMaxDevices];
bool g_ready[kMaxDevices] = {};
std::mutex g_setup_mutex;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Variant of the IBM force-sum kernel (k_ibm_finish) for float32 fields in the reference
// layout: block b reduces cells [b * kNoAllocCellsPerBlock, ...) and markers b, b + grid,
// ...; the last block to finish sums the partials in block order, so the result does not
// depend on scheduling.
__global__ void __launch_bounds__(kNoAllocThreads) k_force_sums_noalloc(
    const float* __restrict__ fx, const float* __restrict__ fy, long long cells,
    const float* __restrict__ FXk, const float* __restrict__ FYk, int n, double* part,
    unsigned int* ticket, double* out) {
    __shared__ double red[kNoAllocThreads / 32][4];
    __shared__ bool last;
    const long long c0 = (long long)blockIdx.x * kNoAllocCellsPerBlock;
    const long long c1 = c0 + kNoAllocCellsPerBlock < cells ? c0 + kNoAllocCellsPerBlock : cells;
    double sx = 0.0, sy = 0.0, mx = 0.0, my = 0.0;
    for (long long c = c0 + threadIdx.x; c < c1; c += kNoAllocThreads) {
        sx += (double)fminf(fmaxf(fx[c], -0.05f), 0.05f);
        sy += (double)fminf(fmaxf(fy[c], -0.05f), 0.05f);
    }
    for (int m = blockIdx.x * kNoAllocThreads + threadIdx.x; m < n; m += gridDim.x * kNoAllocThreads) {
        mx += (double)FXk[m];
        my += (double)FYk[m];
    }
    sx = warp_sum_d(sx); sy = warp_sum_d(sy); mx = warp_sum_d(mx); my = warp_sum_d(my);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { red[warp][0] = sx; red[warp][1] = sy; red[warp][2] = mx; red[warp][3] = my; }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0.0;
        for (int w = 0; w < kNoAllocThreads / 32; ++w) v += red[w][threadIdx.x];
        part[4 * blockIdx.x + threadIdx.x] = v;
        __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (unsigned int b = threadIdx.x; b < gridDim.x; b += kNoAllocThreads)
        for (int e = 0; e < 4; ++e) v[e] += __ldcg(part + 4 * b + e);
    for (int e = 0; e < 4; ++e) v[e] = warp_sum_d(v[e]);
    __syncthreads();
    if (lane == 0)
        for (int e = 0; e < 4; ++e) red[warp][e] = v[e];
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int w = 0; w < kNoAllocThreads / 32; ++w) t += red[w][threadIdx.x];
        out[threadIdx.x] = t;
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

int nfail(int code, const char* msg) {
    clbm::set_last_error(msg);  // reported by clbm_last_error()
    return code;
}

}  // namespace

extern "C" int ibm_force_sums_noalloc(const float* fx, const float* fy, int32_t nx, int32_t ny,
                                      int32_t nz, const float* FXk, const float* FYk, int32_t n,
                                      void* stream, double* out) {
    if (!fx || !fy || !out || nx < 1 || ny < 1 || nz < 1 || n < 0 || (n > 0 && (!FXk || !FYk)))
        return nfail(CLBM_ERR_ARG, "ibm_force_sums_noalloc: invalid argument");
    const long long cells = (long long)nx * ny * nz;
    const long long max_cells = (long long)kNoAllocBlocks * kNoAllocCellsPerBlock;
    if (cells > max_cells) {
        char buf[256];
        snprintf(buf, sizeof(buf),
                 "ibm_force_sums_noalloc: %lld cells exceed the maximum of %lld cells that its "
                 "fixed scratch (%d partial sums) covers", cells, max_cells, kNoAllocBlocks);
        return nfail(CLBM_ERR_ARG, buf);
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return nfail(CLBM_ERR_CUDA, "ibm_force_sums_noalloc: no usable current CUDA device");
    cudaStream_t st = (cudaStream_t)stream;
    // Refuse a stream under capture before issuing anything: the call ends with a copy to
    // host memory and a stream synchronisation, which a capture does not allow. On the
    // legacy default stream the query itself fails while another stream captures in global
    // mode (cudaErrorStreamCaptureImplicit, which leaves that capture valid).
    {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        const cudaError_t qe = cudaStreamIsCapturing(st, &cs);
        if (qe != cudaSuccess) (void)cudaGetLastError();  // the query's own error, not the caller's
        if (qe == cudaErrorStreamCaptureImplicit || (qe == cudaSuccess && cs != cudaStreamCaptureStatusNone))
            return nfail(CLBM_ERR_STATE,
                         "ibm_force_sums_noalloc: the stream is being captured into a CUDA graph; "
                         "the call copies to host memory and waits for the stream, so it must "
                         "run outside capture");
        if (qe != cudaSuccess)
            return nfail(CLBM_ERR_CUDA, "ibm_force_sums_noalloc: cudaStreamIsCapturing failed");
    }
    // One-time set-up per device, with that device current: device addresses of the
    // file-scope scratch, looked up once and kept for the life of the process (so
    // cudaDeviceReset while this library is in use is not supported: the kept addresses
    // would belong to the destroyed context).
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_ready[dev]) {
            Scratch sc;
            if (cudaGetSymbolAddress((void**)&sc.part, g_noalloc_part) != cudaSuccess ||
                cudaGetSymbolAddress((void**)&sc.ticket, g_noalloc_ticket) != cudaSuccess ||
                cudaGetSymbolAddress((void**)&sc.out, g_noalloc_out) != cudaSuccess)
                return nfail(CLBM_ERR_CUDA, "ibm_force_sums_noalloc: cudaGetSymbolAddress failed");
            g_scratch[dev] = sc;
            g_ready[dev] = true;
        }
    }
    const Scratch& sc = g_scratch[dev];
    // An error left pending by the caller's own earlier work is reported as such and left
    // for the caller to read (cudaPeekAtLastError does not clear it).
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess) {
        char buf[256];
        snprintf(buf, sizeof(buf),
                 "ibm_force_sums_noalloc: a CUDA error from earlier work is pending (%s); "
                 "nothing was launched", cudaGetErrorName(pending));
        return nfail(CLBM_ERR_CUDA, buf);
    }
    // The array keeps the last call's contents: clear the ticket that must start at zero.
    if (cudaMemsetAsync(sc.ticket, 0, sizeof(unsigned int), st) != cudaSuccess)
        return nfail(CLBM_ERR_CUDA, "ibm_force_sums_noalloc: cudaMemsetAsync failed");
    const int blocks = (int)((cells + kNoAllocCellsPerBlock - 1) / kNoAllocCellsPerBlock);
    k_force_sums_noalloc<<<blocks, kNoAllocThreads, 0, st>>>(fx, fy, cells, FXk, FYk, n, sc.part,
                                                             sc.ticket, sc.out);
    if (cudaGetLastError() != cudaSuccess)
        return nfail(CLBM_ERR_CUDA, "ibm_force_sums_noalloc: kernel launch failed");
    if (cudaMemcpyAsync(out, sc.out, 4 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return nfail(CLBM_ERR_CUDA, "ibm_force_sums_noalloc: copy of the sums failed");
    return CLBM_OK;
}
