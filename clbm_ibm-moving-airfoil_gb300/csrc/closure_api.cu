// closure_api.cu -- extern "C" entry points of the closure trainer: box-filtered captures
// of a fine lattice, training-sample extraction, sample statistics, loss and gradient
// evaluation, Adam training, and the tensor-core self test.
#include <cstdint>

#include "capi_internal.cuh"

using namespace clbm;
using clbm::api::fail;

struct clbm_trainer {
    int device = 0;
    const clbm_solver* fine = nullptr;   // lattice the captures filter (may be null)
    Grid gc{};                           // coarse lattice (half the fine one)
    float* slot[2] = {nullptr, nullptr}; // filtered pre-collision states
    float* samples = nullptr;            // [closure::kSampleFloats][capacity]
    long long capacity = 0, count = 0;
    float* params = nullptr;             // device working copy of the parameters
    uint16_t* img = nullptr;
    float *part = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
    double* loss = nullptr;              // per-iteration loss sums
    int loss_cap = 0;
    double* stats_part = nullptr;
    double* stats = nullptr;
    long long* cells = nullptr;
    long long cells_cap = 0;
    unsigned int* status = nullptr;
    int grid = 0;                        // training blocks
    cudaStream_t st = nullptr;
};

namespace {

constexpr int kSpin = 1 << 22;           // polls of a bounded mbarrier wait

int tr_sync(clbm_trainer* t) {
    CK(cudaStreamSynchronize(t->st));
    unsigned int status = 0;
    CK(cudaMemcpy(&status, t->status, sizeof(status), cudaMemcpyDeviceToHost));
    if (status) {
        CK(cudaMemset(t->status, 0, sizeof(unsigned int)));
        return fail(CLBM_ERR_STATE, "closure trainer: a bounded tensor-core wait gave up (status %u)", status);
    }
    return CLBM_OK;
}

int ensure_loss(clbm_trainer* t, int n) {
    if (t->loss_cap >= n) return CLBM_OK;
    if (t->loss) CK(cudaFree(t->loss));
    t->loss = nullptr;
    CK(cudaMalloc(&t->loss, sizeof(double) * n));
    t->loss_cap = n;
    return CLBM_OK;
}

int upload_params(clbm_trainer* t, const float* params) {
    CK(cudaMemcpyAsync(t->params, params, sizeof(float) * closure::kParams, cudaMemcpyHostToDevice, t->st));
    launch_closure_images(t->params, t->img, t->st);
    CK_LAUNCH();
    return CLBM_OK;
}

TrainArgs train_args(clbm_trainer* t, long long off, long long count, long long batch, int random,
                     unsigned long long seed, float wscale) {
    TrainArgs a{};
    a.samples = t->samples;
    a.stride = t->capacity;
    a.off = off;
    a.count = count;
    a.batch = batch;
    a.random = random;
    a.seed = seed;
    a.spin_limit = kSpin;
    a.params = t->params;
    a.img = t->img;
    a.wscale = wscale;
    a.part = t->part;
    a.status = t->status;
    return a;
}

int grid_for(const clbm_trainer* t, long long batch) {
    const long long tiles = (batch + 127) / 128;
    return (int)std::max<long long>(1, std::min<long long>(tiles, t->grid));
}

int check_range(const clbm_trainer* t, long long off, long long n, const char* who) {
    if (off < 0 || n <= 0 || off + n > t->count)
        return fail(CLBM_ERR_ARG, "%s: sample range [%lld, %lld) outside [0, %lld)", who, off, off + n, t->count);
    return CLBM_OK;
}

}  // namespace

extern "C" {

int clbm_closure_layout(int32_t* out) {
    if (!out) return fail(CLBM_ERR_ARG, "clbm_closure_layout: null output");
    const int32_t v[] = {closure::kMu, closure::kSinv, closure::kW1, closure::kB1, closure::kW2,
                         closure::kB2, closure::kW3, closure::kB3, closure::kSpan, closure::kParams,
                         closure::kIn, closure::kHid, closure::kTargets, closure::kTrainable,
                         closure::kSampleFloats, closure::kMode, closure::kNu, closure::kSgs,
                         closure::kStats};
    for (int i = 0; i < 19; ++i) out[i] = v[i];
    return CLBM_OK;
}

int clbm_trainer_create(int32_t device, const clbm_solver* fine, int64_t capacity, clbm_trainer** out) {
    if (!out || capacity < 1) return fail(CLBM_ERR_ARG, "clbm_trainer_create: invalid argument");
    *out = nullptr;
    if (fine) {
        if (fine->cfg.storage != CLBM_STORE_F32)
            return fail(CLBM_ERR_ARG, "clbm_trainer_create: the fine lattice must store float32");
        if (fine->g.nx % 2 || fine->g.ny % 2 || fine->g.nz % 2 || fine->g.nx < 8)
            return fail(CLBM_ERR_ARG, "clbm_trainer_create: fine lattice dimensions must be even");
        device = fine->cfg.device;
    }
    CK(cudaSetDevice(device));
    clbm_trainer* t = new clbm_trainer();
    t->device = device;
    t->fine = fine;
    t->capacity = capacity;
    auto bail = [&](int rc) { clbm_trainer_destroy(t); return rc; };
    if (cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking) != cudaSuccess)
        return bail(fail(CLBM_ERR_CUDA, "clbm_trainer_create: stream creation failed"));
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    t->grid = std::max(sms, 1);
    const size_t samples = sizeof(float) * closure::kSampleFloats * (size_t)capacity;
    if (cudaMalloc(&t->samples, samples) != cudaSuccess ||
        cudaMalloc(&t->params, sizeof(float) * closure::kParams) != cudaSuccess ||
        cudaMalloc(&t->img, sizeof(uint16_t) * closure::kImgElems) != cudaSuccess ||
        cudaMalloc(&t->part, sizeof(float) * closure_part_floats() * t->grid) != cudaSuccess ||
        cudaMalloc(&t->grad, sizeof(float) * closure::kTrainable) != cudaSuccess ||
        cudaMalloc(&t->m1, sizeof(float) * closure::kTrainable) != cudaSuccess ||
        cudaMalloc(&t->m2, sizeof(float) * closure::kTrainable) != cudaSuccess ||
        cudaMalloc(&t->stats_part, sizeof(double) * closure::kStats * 1024) != cudaSuccess ||
        cudaMalloc(&t->stats, sizeof(double) * closure::kStats) != cudaSuccess ||
        cudaMalloc(&t->status, sizeof(unsigned int)) != cudaSuccess ||
        cudaMemset(t->status, 0, sizeof(unsigned int)) != cudaSuccess)
        return bail(fail(CLBM_ERR_CUDA, "clbm_trainer_create: device allocation failed"));
    if (fine) {
        Grid& g = t->gc;
        g.nx = fine->g.nx / 2;
        g.ny = fine->g.ny / 2;
        g.nz = fine->g.nz / 2;
        g.pitch = (g.nx + 31) / 32 * 32;
        g.plane = (long long)g.pitch * g.ny * g.nz;
        g.status = t->status;
        const size_t bytes = sizeof(float) * (19 + closure::kAux) * (size_t)g.plane;
        for (int k = 0; k < 2; ++k)
            if (cudaMalloc(&t->slot[k], bytes) != cudaSuccess)
                return bail(fail(CLBM_ERR_CUDA, "clbm_trainer_create: device allocation failed"));
    }
    *out = t;
    return CLBM_OK;
}

int clbm_trainer_destroy(clbm_trainer* t) {
    if (!t) return CLBM_OK;
    if (t->st) cudaStreamSynchronize(t->st);
    void* ptrs[] = {t->slot[0], t->slot[1], t->samples, t->params, t->img, t->part, t->grad, t->m1,
                    t->m2, t->loss, t->stats_part, t->stats, t->cells, t->status};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (t->st) cudaStreamDestroy(t->st);
    delete t;
    return CLBM_OK;
}

int clbm_trainer_capture(clbm_trainer* t, int32_t slot) {
    if (!t || slot < 0 || slot > 1) return fail(CLBM_ERR_ARG, "clbm_trainer_capture: invalid argument");
    if (!t->fine) return fail(CLBM_ERR_STATE, "clbm_trainer_capture: trainer has no fine lattice");
    const clbm_solver* s = t->fine;
    CK(cudaSetDevice(t->device));
    // the fine solver's queued steps come first
    CK(cudaStreamSynchronize(s->st));
    CK(cudaStreamSynchronize(s->st2));
    launch_filter2(!s->local, (const float*)s->f[s->cur], s->g, s->c, t->slot[slot], t->gc, t->st);
    CK_LAUNCH();
    return tr_sync(t);
}

int clbm_trainer_read_slot(clbm_trainer* t, int32_t slot, float* out) {
    if (!t || slot < 0 || slot > 1 || !out || !t->slot[0])
        return fail(CLBM_ERR_ARG, "clbm_trainer_read_slot: invalid argument");
    const Grid& g = t->gc;
    constexpr int nch = 19 + closure::kAux;
    std::vector<float> h((size_t)nch * g.plane);
    CK(cudaMemcpy(h.data(), t->slot[slot], sizeof(float) * h.size(), cudaMemcpyDeviceToHost));
    // reference layout (nx, ny, nz, 28), z fastest: 19 populations, then the filtered
    // velocity (3) and velocity products (xx, yy, zz, xy, xz, yz)
    for (int x = 0; x < g.nx; ++x)
        for (int y = 0; y < g.ny; ++y)
            for (int z = 0; z < g.nz; ++z)
                for (int q = 0; q < nch; ++q)
                    out[(((size_t)x * g.ny + y) * g.nz + z) * nch + q] =
                        h[(size_t)q * g.plane + ((size_t)z * g.ny + y) * g.pitch + x];
    return CLBM_OK;
}

int clbm_trainer_extract(clbm_trainer* t, const int64_t* cells, int64_t n) {
    if (!t || !cells || n < 1) return fail(CLBM_ERR_ARG, "clbm_trainer_extract: invalid argument");
    if (!t->fine) return fail(CLBM_ERR_STATE, "clbm_trainer_extract: trainer has no fine lattice");
    if (t->count + n > t->capacity)
        return fail(CLBM_ERR_ARG, "clbm_trainer_extract: %lld samples exceed the capacity %lld",
                    (long long)(t->count + n), t->capacity);
    const Grid& g = t->gc;
    const long long total = (long long)g.nx * g.ny * g.nz;
    for (int64_t j = 0; j < n; ++j) {
        const long long x = cells[j] % g.nx;
        if (cells[j] < 0 || cells[j] >= total || x < 1 || x > g.nx - 2)
            return fail(CLBM_ERR_ARG, "clbm_trainer_extract: cell %lld outside 1 <= x <= nx - 2", (long long)cells[j]);
    }
    CK(cudaSetDevice(t->device));
    if (t->cells_cap < n) {
        if (t->cells) CK(cudaFree(t->cells));
        t->cells = nullptr;
        CK(cudaMalloc(&t->cells, sizeof(long long) * n));
        t->cells_cap = n;
    }
    CK(cudaMemcpyAsync(t->cells, cells, sizeof(long long) * n, cudaMemcpyHostToDevice, t->st));
    launch_closure_samples(t->slot[0], t->slot[1], g, t->cells, n, t->samples, t->capacity, t->count, t->st);
    CK_LAUNCH();
    if (int rc = tr_sync(t)) return rc;
    t->count += n;
    return CLBM_OK;
}

int clbm_trainer_count(const clbm_trainer* t, int64_t* n) {
    if (!t || !n) return fail(CLBM_ERR_ARG, "clbm_trainer_count: invalid argument");
    *n = t->count;
    return CLBM_OK;
}

int clbm_trainer_write_samples(clbm_trainer* t, int64_t off, int64_t n, const float* in) {
    if (!t || !in || off < 0 || n < 1 || off + n > t->capacity)
        return fail(CLBM_ERR_ARG, "clbm_trainer_write_samples: invalid argument");
    CK(cudaSetDevice(t->device));
    std::vector<float> col((size_t)n);
    for (int i = 0; i < closure::kSampleFloats; ++i) {
        for (int64_t j = 0; j < n; ++j) col[(size_t)j] = in[(size_t)j * closure::kSampleFloats + i];
        CK(cudaMemcpy(t->samples + (size_t)i * t->capacity + off, col.data(), sizeof(float) * (size_t)n,
                      cudaMemcpyHostToDevice));
    }
    if (int rc = tr_sync(t)) return rc;
    t->count = std::max<long long>(t->count, off + n);
    return CLBM_OK;
}

int clbm_trainer_read_samples(clbm_trainer* t, int64_t off, int64_t n, float* out) {
    if (!t || !out) return fail(CLBM_ERR_ARG, "clbm_trainer_read_samples: invalid argument");
    if (int rc = check_range(t, off, n, "clbm_trainer_read_samples")) return rc;
    CK(cudaSetDevice(t->device));
    if (int rc = tr_sync(t)) return rc;
    std::vector<float> col((size_t)n);
    for (int i = 0; i < closure::kSampleFloats; ++i) {
        CK(cudaMemcpy(col.data(), t->samples + (size_t)i * t->capacity + off, sizeof(float) * (size_t)n,
                      cudaMemcpyDeviceToHost));
        for (int64_t j = 0; j < n; ++j) out[(size_t)j * closure::kSampleFloats + i] = col[(size_t)j];
    }
    return CLBM_OK;
}

int clbm_trainer_stats(clbm_trainer* t, int64_t off, int64_t n, double* out) {
    if (!t || !out) return fail(CLBM_ERR_ARG, "clbm_trainer_stats: invalid argument");
    if (int rc = check_range(t, off, n, "clbm_trainer_stats")) return rc;
    CK(cudaSetDevice(t->device));
    const int blocks = (int)std::min<long long>(1024, (n + 255) / 256);
    launch_sample_stats(t->samples + off, t->capacity, n, t->stats_part, blocks, t->stats, t->st);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(out, t->stats, sizeof(double) * closure::kStats, cudaMemcpyDeviceToHost, t->st));
    return tr_sync(t);
}

int clbm_trainer_loss(clbm_trainer* t, const float* params, int64_t off, int64_t n, float wscale,
                      double* loss_sum) {
    if (!t || !params || !loss_sum) return fail(CLBM_ERR_ARG, "clbm_trainer_loss: invalid argument");
    if (int rc = check_range(t, off, n, "clbm_trainer_loss")) return rc;
    CK(cudaSetDevice(t->device));
    if (int rc = ensure_loss(t, 1)) return rc;
    if (int rc = upload_params(t, params)) return rc;
    const TrainArgs a = train_args(t, off, n, n, 0, 0, wscale);
    const int grid = grid_for(t, n);
    launch_closure_train(a, false, grid, t->st);
    CK_LAUNCH();
    launch_closure_reduce(t->part, grid, 1.0f / (float)n, t->grad, t->loss, t->st);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(loss_sum, t->loss, sizeof(double), cudaMemcpyDeviceToHost, t->st));
    return tr_sync(t);
}

int clbm_trainer_grad(clbm_trainer* t, const float* params, int64_t off, int64_t n, float wscale,
                      float* grad, double* loss_sum) {
    if (!t || !params || !grad || !loss_sum) return fail(CLBM_ERR_ARG, "clbm_trainer_grad: invalid argument");
    if (int rc = check_range(t, off, n, "clbm_trainer_grad")) return rc;
    CK(cudaSetDevice(t->device));
    if (int rc = ensure_loss(t, 1)) return rc;
    if (int rc = upload_params(t, params)) return rc;
    const TrainArgs a = train_args(t, off, n, n, 0, 0, wscale);
    const int grid = grid_for(t, n);
    launch_closure_train(a, true, grid, t->st);
    CK_LAUNCH();
    launch_closure_reduce(t->part, grid, 1.0f / (float)n, t->grad, t->loss, t->st);
    CK_LAUNCH();
    CK(cudaMemcpyAsync(grad, t->grad, sizeof(float) * closure::kTrainable, cudaMemcpyDeviceToHost, t->st));
    CK(cudaMemcpyAsync(loss_sum, t->loss, sizeof(double), cudaMemcpyDeviceToHost, t->st));
    return tr_sync(t);
}

int clbm_trainer_fit(clbm_trainer* t, float* params, int64_t off, int64_t n, int32_t iters, int64_t batch,
                     float lr, float wscale, uint64_t seed, double* loss_hist) {
    if (!t || !params || iters < 1 || batch < 1) return fail(CLBM_ERR_ARG, "clbm_trainer_fit: invalid argument");
    if (int rc = check_range(t, off, n, "clbm_trainer_fit")) return rc;
    CK(cudaSetDevice(t->device));
    if (int rc = ensure_loss(t, iters)) return rc;
    if (int rc = upload_params(t, params)) return rc;
    CK(cudaMemsetAsync(t->m1, 0, sizeof(float) * closure::kTrainable, t->st));
    CK(cudaMemsetAsync(t->m2, 0, sizeof(float) * closure::kTrainable, t->st));
    const int grid = grid_for(t, batch);
    for (int it = 0; it < iters; ++it) {
        // cosine decay of the learning rate to zero
        const float lrt = 0.5f * lr * (1.0f + cosf(3.14159265f * (float)it / (float)iters));
        const TrainArgs a = train_args(t, off, n, batch, 1, seed + 0x9E3779B97F4A7C15ull * (uint64_t)(it + 1), wscale);
        launch_closure_train(a, true, grid, t->st);
        launch_closure_reduce(t->part, grid, 1.0f / (float)batch, t->grad, t->loss + it, t->st);
        launch_closure_adam(t->params, t->grad, t->m1, t->m2, lrt, 0.9f, 0.999f, 1e-8f, it + 1, t->st);
        launch_closure_images(t->params, t->img, t->st);
        CK_LAUNCH();
    }
    CK(cudaMemcpyAsync(params, t->params, sizeof(float) * closure::kParams, cudaMemcpyDeviceToHost, t->st));
    if (loss_hist)
        CK(cudaMemcpyAsync(loss_hist, t->loss, sizeof(double) * iters, cudaMemcpyDeviceToHost, t->st));
    return tr_sync(t);
}

int clbm_tc_selftest(int32_t device, const float* A, const float* B, float* D, int32_t kdim, int32_t n) {
    if (!A || !B || !D || (kdim != 32 && kdim != 128) || (n != 32 && n != 112))
        return fail(CLBM_ERR_ARG, "clbm_tc_selftest: invalid argument");
    CK(cudaSetDevice(device));
    float *dA = nullptr, *dB = nullptr, *dD = nullptr;
    unsigned int* st = nullptr;
    auto cleanup = [&]() {
        if (dA) cudaFree(dA);
        if (dB) cudaFree(dB);
        if (dD) cudaFree(dD);
        if (st) cudaFree(st);
    };
    if (cudaMalloc(&dA, sizeof(float) * 128 * kdim) != cudaSuccess ||
        cudaMalloc(&dB, sizeof(float) * n * kdim) != cudaSuccess ||
        cudaMalloc(&dD, sizeof(float) * 128 * n) != cudaSuccess ||
        cudaMalloc(&st, sizeof(unsigned int)) != cudaSuccess) {
        cleanup();
        return fail(CLBM_ERR_CUDA, "clbm_tc_selftest: allocation failed");
    }
    cudaMemcpy(dA, A, sizeof(float) * 128 * kdim, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B, sizeof(float) * n * kdim, cudaMemcpyHostToDevice);
    cudaMemset(st, 0, sizeof(unsigned int));
    launch_tc_selftest(dA, dB, dD, kdim, n, st, kSpin, nullptr);
    cudaError_t e = cudaDeviceSynchronize();
    unsigned int status = 0;
    if (e == cudaSuccess) e = cudaMemcpy(D, dD, sizeof(float) * 128 * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&status, st, sizeof(status), cudaMemcpyDeviceToHost);
    cleanup();
    if (e != cudaSuccess) return fail(CLBM_ERR_CUDA, "clbm_tc_selftest: %s", cudaGetErrorString(e));
    if (status) return fail(CLBM_ERR_STATE, "clbm_tc_selftest: bounded wait gave up");
    return CLBM_OK;
}

}  // extern "C"
