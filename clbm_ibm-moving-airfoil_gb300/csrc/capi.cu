// capi.cu -- extern "C" entry points (include/clbm_gb300.h): object lifetimes, host-side
// sequencing of the kernels on the solver's stream, CUDA-graph capture of the time loop,
// transfers in the reference layout and error reporting.
#include "capi_internal.cuh"

using namespace clbm;
using clbm::api::fail;

namespace {

thread_local std::string g_err;

constexpr double kWd[19] = {1.0 / 3,  1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18,
                            1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                            1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};
constexpr int kHistCap = CLBM_HISTORY_CAPACITY;
// kernels one graph-captured step launches: markers, band-prepare, interp/spread, bulk
// stream-collide, box stream-collide with the force sums
constexpr int kKernelsPerIbmStep = 5;
// steps per captured graph (even, so buffer and box-slot parities repeat); within a graph
// each step's marker kernel overlaps the previous step's bulk pass
constexpr int kGraphSteps = 8;
// density floor of the divergence monitor: main_moving.py:143 stops below rho = 0.3
constexpr double kRhoFloor = 0.3;
// graph replays clbm_run keeps in flight; it reads the status word of the oldest one
constexpr int kReplaysInFlight = 4;

}  // namespace

int clbm::api::fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

void clbm::set_last_error(const char* msg) { g_err = msg; }

namespace {

int ensure_stage(clbm_solver* s, size_t bytes) {
    if (s->stage_bytes >= bytes) return CLBM_OK;
    if (s->stage) CK(cudaFree(s->stage));
    s->stage = nullptr;
    s->stage_bytes = 0;
    CK(cudaMalloc(&s->stage, bytes));
    s->stage_bytes = bytes;
    return CLBM_OK;
}

size_t cells(const clbm_solver* s) { return (size_t)s->g.nx * s->g.ny * s->g.nz; }

int record_event(clbm_solver* s, cudaStream_t st) {
    if (s->ev_used == s->ev.size()) {
        cudaEvent_t e;
        CK(cudaEventCreate(&e));
        s->ev.push_back(e);
    }
    CK(cudaEventRecord(s->ev[s->ev_used++], st));
    return CLBM_OK;
}

// Make the main stream wait for a bulk pass that a step left running on the second stream.
int join_bulk(clbm_solver* s) {
    if (s->bulk_pending) {
        CK(cudaStreamWaitEvent(s->st, s->ev_bulk, 0));
        s->bulk_pending = false;
    }
    return CLBM_OK;
}

// Box pass of an IBM step on stream st: with the force sums of the IBM call when they are
// still pending (no separate force-sum kernel then).
void box_pass(clbm_solver* s, const ForceArgs& fa, const clbm_ibm* ibm, cudaStream_t st) {
    if (ibm->sums_pending) {
        launch_stream_collide_box_sums(s->cfg.storage, !s->local, s->f[s->cur], s->f[1 - s->cur],
                                       s->g, s->c, fa, ibm->a, st);
        ibm->sums_pending = false;
    } else {
        launch_stream_collide_box(s->cfg.storage, !s->local, s->f[s->cur], s->f[1 - s->cur], s->g,
                                  s->c, fa, ibm->a.max_bx, ibm->a.max_by, ibm->a.max_bz, st);
    }
}

// One fused stream-collide launch on stream `st`, bracketed by timing events if profiling.
int sc_timed(clbm_solver* s, int fmode, const ForceArgs& fa, cudaStream_t st, bool box,
             const clbm_ibm* ibm = nullptr) {
    if (s->prof) {
        if (int rc = record_event(s, st)) return rc;
        s->ev_tag.resize(s->ev_used / 2 + 1);
        s->ev_tag[s->ev_used / 2] = box ? 1 : 0;
    }
    if (box) {
        box_pass(s, fa, ibm, st);
    } else if (s->closure && (fmode == kForceNone || fmode == kForceSkipBand)) {
        ClosureArgs ca{};
        ca.params = s->cl_params;
        ca.img = s->cl_img;
        ca.cells = (long long)cells(s);
        launch_closure_stream_collide(s->cfg.storage, !s->local, fmode, s->f[s->cur], s->f[1 - s->cur],
                                      s->g, s->c, fa, ca, s->cl_grid, st);
    } else {
        launch_stream_collide(s->cfg.storage, !s->local, fmode, s->variant, s->f[s->cur],
                              s->f[1 - s->cur], s->g, s->c, fa, st);
    }
    CK_LAUNCH();
    if (s->prof)
        if (int rc = record_event(s, st)) return rc;
    s->launches += 1;
    return CLBM_OK;
}

// Force sums of an IBM call that no step has completed yet, by the force-sum kernel (needed
// when the history is read, or another compute_force comes, before the next step).
int flush_sums(const clbm_ibm* ibm) {
    if (!ibm->sums_pending) return CLBM_OK;
    launch_ibm_finish(ibm->a, ibm->s->g, ibm->s->st);
    CK_LAUNCH();
    ibm->s->launches += 1;
    ibm->sums_pending = false;
    return CLBM_OK;
}

int step_impl(clbm_solver* s, int fmode, const ForceArgs& fa, const clbm_ibm* ibm) {
    if (int rc = join_bulk(s)) return rc;
    if (fmode != kForceBand) {
        if (int rc = sc_timed(s, fmode, fa, s->st, false)) return rc;
    } else {
        // IBM step in two passes. The bulk pass (cells outside the force box) needs only the
        // box, so it forks off after the marker kernel of the last compute_force and runs on
        // the low-priority stream while the IBM chain still computes the forces; the box
        // pass follows the IBM chain on the main stream; the main stream then joins the
        // bulk pass. The fork is valid only while the state is the one compute_force saw.
        // CLBM_SERIAL=1: both passes on the main stream after the IBM chain, one after the
        // other (the bulk pass then runs alone: its isolated time for measurements)
        static const int serial = knob("CLBM_SERIAL", 0);
        if (serial) {
            if (int rc = sc_timed(s, kForceSkipBand, fa, s->st, false)) return rc;
            if (int rc = sc_timed(s, kForceBand, fa, s->st, true, ibm)) return rc;
            s->cur = 1 - s->cur;
            s->local = false;
            s->macro_full = false;
            s->version += 1;
            return CLBM_OK;
        }
        if (ibm->box_version == s->version) {
            CK(cudaStreamWaitEvent(s->st2, ibm->ev_box, 0));
        } else {
            CK(cudaEventRecord(s->ev_fork, s->st));
            CK(cudaStreamWaitEvent(s->st2, s->ev_fork, 0));
        }
        if (int rc = sc_timed(s, kForceSkipBand, fa, s->st2, false)) return rc;
        CK(cudaEventRecord(s->ev_bulk, s->st2));
        if (int rc = sc_timed(s, kForceBand, fa, s->st, true, ibm)) return rc;
        s->bulk_pending = true;  // joined by the next call (after the next marker kernel)
    }
    s->cur = 1 - s->cur;
    s->local = false;
    s->macro_full = false;
    s->version += 1;
    return CLBM_OK;
}

int ibm_force_impl(clbm_ibm* ibm, bool devm, const MotionF& mf, const clbm_motion& m) {
    clbm_solver* s = ibm->s;
    // a previous call that no step completed: its sums first (they advance the counter)
    if (int rc = flush_sums(ibm)) return rc;
    // the marker kernel needs only the motion: it runs beside the previous step's bulk pass
    launch_ibm_markers(ibm->a, s->g, devm, mf, m, s->st);
    CK(cudaEventRecord(ibm->ev_box, s->st));
    if (int rc = join_bulk(s)) return rc;
    ibm->box_version = s->version;
    launch_band_prepare(s->cfg.storage, !s->local, s->f[s->cur], s->g, s->c, ibm->a.dev,
                        ibm->a.fx, ibm->a.fy, s->rho, s->ux, s->uy, s->uz, ibm->a.max_bx,
                        ibm->a.max_by, ibm->a.max_bz, !s->macro_full, s->st);
    launch_ibm_interp_spread(ibm->a, s->g, s->st);
    CK_LAUNCH();
    s->launches += (ibm->a.n > 0) ? 3 : 1;
    // the force sums of this call are computed by the box pass of the next step
    ibm->sums_pending = true;
    ibm->calls += 1;
    return CLBM_OK;
}

// Full-grid kernel variant: CLBM_KERNEL=cell|pair|staged forces one; otherwise lattices of
// at least 2^20 cells time each candidate (three launches after one warm-up, on the
// not-yet-initialised buffers) and keep the fastest; smaller lattices use the staged one.
int pick_variant(clbm_solver* s) {
    const bool half = s->cfg.storage != CLBM_STORE_F32;
    if (const char* env = std::getenv("CLBM_KERNEL")) {
        if (!std::strcmp(env, "cell")) return kVariantCell;
        if (!std::strcmp(env, "pair") && half) return kVariantPair;
        if (!std::strcmp(env, "staged")) return kVariantStaged;
    }
    const long long n = (long long)s->g.nx * s->g.ny * s->g.nz;
    if (n < (1LL << 20)) return kVariantStaged;
    // Candidates in order of preference under load: the staged kernel holds more registers
    // and shared memory per cell and loses more when the IBM kernels share the SMs, so a
    // later candidate must be at least 3 % faster in isolation to be chosen.
    std::vector<int> cand = {kVariantCell};
    if (half) cand.push_back(kVariantPair);
    cand.push_back(kVariantStaged);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return kVariantStaged;
    if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); return kVariantStaged; }
    int best = kVariantStaged;
    float best_ms = 1e30f;
    for (int v : cand) {
        ForceArgs fa{};
        launch_stream_collide(s->cfg.storage, true, kForceNone, v, s->f[0], s->f[1], s->g, s->c, fa, s->st);
        cudaEventRecord(e0, s->st);
        for (int k = 0; k < 3; ++k)
            launch_stream_collide(s->cfg.storage, true, kForceNone, v, s->f[k & 1], s->f[1 - (k & 1)],
                                  s->g, s->c, fa, s->st);
        cudaEventRecord(e1, s->st);
        float ms = 0.f;
        if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) {
            s->variant_ms[v] = ms / 3.0f;
            if (ms < 0.97f * best_ms) {
                best_ms = ms;
                best = v;
            }
        }
        s->launches += 4;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGetLastError();
    return best;
}

void free_graph(clbm_solver* s) {
    if (s->gexec) cudaGraphExecDestroy(s->gexec);
    s->gexec = nullptr;
    s->g_ibm = nullptr;
    s->g_cur = -1;
    s->g_slot = -1;
}

}  // namespace

extern "C" {

const char* clbm_last_error(void) { return g_err.c_str(); }

int clbm_create(const clbm_config* cfg, clbm_solver** out) {
    if (!cfg || !out) return fail(CLBM_ERR_ARG, "clbm_create: null argument");
    *out = nullptr;
    if (cfg->nx < 3 || cfg->ny < 1 || cfg->nz < 1)
        return fail(CLBM_ERR_ARG, "clbm_create: lattice %dx%dx%d invalid (nx >= 3, ny, nz >= 1)",
                    cfg->nx, cfg->ny, cfg->nz);
    if (cfg->storage < CLBM_STORE_F32 || cfg->storage > CLBM_STORE_BF16S)
        return fail(CLBM_ERR_ARG, "clbm_create: unknown storage %d", cfg->storage);
    if (!(cfg->s_v > 0.0 && cfg->s_v < 2.0))
        return fail(CLBM_ERR_ARG, "clbm_create: s_v = %g outside (0, 2)", cfg->s_v);
    const long long pitch = ((long long)cfg->nx + 31) / 32 * 32;
    const long long plane = pitch * cfg->ny * cfg->nz;
    if (plane * 19 >= (1LL << 40))
        return fail(CLBM_ERR_ARG, "clbm_create: lattice too large");
    if (cudaSetDevice(cfg->device) != cudaSuccess)
        return fail(CLBM_ERR_CUDA, "clbm_create: cannot use CUDA device %d: %s", cfg->device,
                    cudaGetErrorString(cudaGetLastError()));
    clbm_solver* s = new clbm_solver();
    s->cfg = *cfg;
    s->g.nx = cfg->nx; s->g.ny = cfg->ny; s->g.nz = cfg->nz;
    s->g.pitch = (int)pitch; s->g.plane = plane;
    s->g.seg = staged_segment(cfg->nx);
    s->g.spin_limit = 1 << 22;
    s->g.extra_tx = 0;
    s->c.one_m_sv = (float)(1.0 - cfg->s_v);
    s->c.s_e = (float)cfg->s_e;
    s->c.ux_in = (float)cfg->ux_in;
    s->c.uy_in = (float)cfg->uy_in;
    s->c.c23 = (float)(2.0 / 3.0);
    s->c.c16 = (float)(1.0 / 6.0);
    for (int q = 0; q < 19; ++q) s->c.wc[q] = (float)(kWd[q] * (1.0 - cfg->s_v * 0.5));
    s->c.rho_floor = (float)kRhoFloor;
    s->c.status = nullptr;  // monitor off while the variants are timed on zeroed buffers
    auto bail = [&](int rc) { clbm_destroy(s); return rc; };
    int prio_low = 0, prio_high = 0;
    cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (cudaStreamCreateWithPriority(&s->st, cudaStreamNonBlocking, prio_high) != cudaSuccess ||
        cudaStreamCreateWithPriority(&s->st2, cudaStreamNonBlocking, prio_low) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_bulk, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(CLBM_ERR_CUDA, "clbm_create: no CUDA device or stream creation failed: %s",
                         cudaGetErrorString(cudaGetLastError())));
    const size_t fbytes = (size_t)plane * 19 * store_bytes(cfg->storage);
    for (int b = 0; b < 2; ++b) {
        if (cudaMalloc(&s->f[b], fbytes) != cudaSuccess)
            return bail(fail(CLBM_ERR_CUDA, "clbm_create: cudaMalloc of %zu bytes failed", fbytes));
        cudaMemsetAsync(s->f[b], 0, fbytes, s->st);
    }
    float** fields[] = {&s->rho, &s->ux, &s->uy, &s->uz};
    for (float** p : fields) {
        if (cudaMalloc(p, (size_t)plane * sizeof(float)) != cudaSuccess)
            return bail(fail(CLBM_ERR_CUDA, "clbm_create: cudaMalloc of macro field failed"));
        cudaMemsetAsync(*p, 0, (size_t)plane * sizeof(float), s->st);
    }
    if (cudaMalloc(&s->stats, 4 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&s->status, sizeof(unsigned int)) != cudaSuccess)
        return bail(fail(CLBM_ERR_CUDA, "clbm_create: cudaMalloc failed"));
    cudaMemsetAsync(s->status, 0, sizeof(unsigned int), s->st);
    s->g.status = s->status;
    s->variant = pick_variant(s);
    s->c.status = s->status;
    if (cudaHostAlloc((void**)&s->h_status, sizeof(unsigned int), cudaHostAllocDefault) != cudaSuccess)
        return bail(fail(CLBM_ERR_CUDA, "clbm_create: pinned allocation failed"));
    *s->h_status = 0;
    for (cudaEvent_t& e : s->ev_replay)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
            return bail(fail(CLBM_ERR_CUDA, "clbm_create: event creation failed"));
    launch_init(cfg->storage, s->f[0], s->g, s->c, s->st);
    launch_fill_macro(s->g, s->c, s->rho, s->ux, s->uy, s->uz, s->st);
    s->launches += 2;
    s->cur = 0;
    s->local = true;
    s->macro_full = true;
    cudaError_t e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess)
        return bail(fail(CLBM_ERR_CUDA, "clbm_create: %s", cudaGetErrorString(e)));
    *out = s;
    return CLBM_OK;
}

int clbm_destroy(clbm_solver* s) {
    if (!s) return CLBM_OK;
    if (s->st) cudaStreamSynchronize(s->st);
    if (s->st2) cudaStreamSynchronize(s->st2);
    free_graph(s);
    for (clbm_ibm* ibm : s->ibms) ibm->s = nullptr;
    s->ibms.clear();
    for (cudaEvent_t e : s->ev) cudaEventDestroy(e);
    void* ptrs[] = {s->f[0], s->f[1], s->rho, s->ux, s->uy, s->uz, s->dfx, s->dfy, s->dfz,
                    s->stage, s->stats, s->status, s->cl_params, s->cl_img};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (s->ev_bulk) cudaEventDestroy(s->ev_bulk);
    if (s->ev_fork) cudaEventDestroy(s->ev_fork);
    for (cudaEvent_t e : s->ev_replay)
        if (e) cudaEventDestroy(e);
    if (s->h_status) cudaFreeHost(s->h_status);
    if (s->st2) cudaStreamDestroy(s->st2);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
    return CLBM_OK;
}

int clbm_step(clbm_solver* s, const clbm_ibm* ibm) {
    if (!s) return fail(CLBM_ERR_ARG, "clbm_step: null solver");
    if (ibm && ibm->s != s) return fail(CLBM_ERR_ARG, "clbm_step: IBM bound to another solver");
    ForceArgs fa{};
    if (ibm) {
        fa.qx = ibm->a.fx;
        fa.qy = ibm->a.fy;
        fa.dev = ibm->a.dev;
        fa.slot = (int)(ibm->calls & 1);  // box of the last compute_force call
    }
    return step_impl(s, ibm ? kForceBand : kForceNone, fa, ibm);
}

int clbm_step_dense_force(clbm_solver* s, const float* fx, const float* fy, const float* fz) {
    if (!s || !fx || !fy) return fail(CLBM_ERR_ARG, "clbm_step_dense_force: null argument");
    const size_t pb = (size_t)s->g.plane * sizeof(float);
    float** bufs[] = {&s->dfx, &s->dfy, &s->dfz};
    for (float** p : bufs)
        if (!*p) {
            CK(cudaMalloc(p, pb));
            CK(cudaMemsetAsync(*p, 0, pb, s->st));
        }
    launch_import_field(fx, s->dfx, s->g, s->st);
    launch_import_field(fy, s->dfy, s->g, s->st);
    if (fz) launch_import_field(fz, s->dfz, s->g, s->st);
    else CK(cudaMemsetAsync(s->dfz, 0, pb, s->st));
    CK_LAUNCH();
    s->launches += fz ? 3 : 2;
    ForceArgs fa{s->dfx, s->dfy, s->dfz, nullptr, nullptr, nullptr};
    return step_impl(s, kForceDense, fa, nullptr);
}

int clbm_step_host_force(clbm_solver* s, const float* fx, const float* fy, const float* fz) {
    if (!s || !fx || !fy) return fail(CLBM_ERR_ARG, "clbm_step_host_force: null argument");
    const size_t n = cells(s);
    int rc = ensure_stage(s, 3 * n * sizeof(float));
    if (rc) return rc;
    CK(cudaMemcpyAsync(s->stage, fx, n * sizeof(float), cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(s->stage + n, fy, n * sizeof(float), cudaMemcpyHostToDevice, s->st));
    if (fz) CK(cudaMemcpyAsync(s->stage + 2 * n, fz, n * sizeof(float), cudaMemcpyHostToDevice, s->st));
    rc = clbm_step_dense_force(s, s->stage, s->stage + n, fz ? s->stage + 2 * n : nullptr);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->st));  // the host arrays may be released after return
    return CLBM_OK;
}

static int materialize(clbm_solver* s, bool with_stats) {
    if (with_stats) {
        unsigned long long init[4] = {~0ull, 0ull, 0ull, 0ull};
        CK(cudaMemcpyAsync(s->stats, init, sizeof(init), cudaMemcpyHostToDevice, s->st));
    }
    if (!s->macro_full || with_stats) {
        launch_macro_full(s->cfg.storage, !s->local, s->f[s->cur], s->g, s->c, s->rho, s->ux,
                          s->uy, s->uz, with_stats ? s->stats : nullptr, s->st);
        CK_LAUNCH();
        s->launches += 1;
        s->macro_full = true;
    }
    return CLBM_OK;
}

int clbm_read_macro(clbm_solver* s, float* rho, float* ux, float* uy, float* uz) {
    if (!s) return fail(CLBM_ERR_ARG, "clbm_read_macro: null solver");
    if (int rc = join_bulk(s)) return rc;
    int rc = materialize(s, false);
    if (rc) return rc;
    const size_t n = cells(s);
    rc = ensure_stage(s, 4 * n * sizeof(float));
    if (rc) return rc;
    const float* src[4] = {s->rho, s->ux, s->uy, s->uz};
    float* dst[4] = {rho, ux, uy, uz};
    for (int k = 0; k < 4; ++k) {
        if (!dst[k]) continue;
        launch_export_field(src[k], s->stage + k * n, s->g, 0.0f, s->st);
        CK_LAUNCH();
        s->launches += 1;
        CK(cudaMemcpyAsync(dst[k], s->stage + k * n, n * sizeof(float), cudaMemcpyDeviceToHost,
                           s->st));
    }
    CK(cudaStreamSynchronize(s->st));
    return CLBM_OK;
}

int clbm_read_vorticity_slice(clbm_solver* s, int32_t z, float* out) {
    if (!s || !out || z < 0 || z >= s->g.nz)
        return fail(CLBM_ERR_ARG, "clbm_read_vorticity_slice: invalid argument");
    if (int rc = join_bulk(s)) return rc;
    int rc = materialize(s, false);
    if (rc) return rc;
    const size_t n = (size_t)s->g.nx * s->g.ny;
    rc = ensure_stage(s, n * sizeof(float));
    if (rc) return rc;
    launch_vorticity_slice(s->ux, s->uy, s->g, z, s->stage, s->st);
    CK_LAUNCH();
    s->launches += 1;
    CK(cudaMemcpyAsync(out, s->stage, n * sizeof(float), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    return CLBM_OK;
}

int clbm_read_populations(clbm_solver* s, float* f_host) {
    if (!s || !f_host) return fail(CLBM_ERR_ARG, "clbm_read_populations: null argument");
    if (int rc = join_bulk(s)) return rc;
    const size_t n = cells(s) * 19;
    int rc = ensure_stage(s, n * sizeof(float));
    if (rc) return rc;
    launch_export_populations(s->cfg.storage, !s->local, s->f[s->cur], s->stage, s->g, s->c,
                              s->st);
    CK_LAUNCH();
    s->launches += 1;
    CK(cudaMemcpyAsync(f_host, s->stage, n * sizeof(float), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    return CLBM_OK;
}

int clbm_write_populations(clbm_solver* s, const float* f_host) {
    if (!s || !f_host) return fail(CLBM_ERR_ARG, "clbm_write_populations: null argument");
    if (int rc = join_bulk(s)) return rc;
    const size_t n = cells(s) * 19;
    int rc = ensure_stage(s, n * sizeof(float));
    if (rc) return rc;
    CK(cudaMemcpyAsync(s->stage, f_host, n * sizeof(float), cudaMemcpyHostToDevice, s->st));
    launch_import_populations(s->cfg.storage, s->stage, s->f[s->cur], s->g, s->st);
    CK_LAUNCH();
    // a new state: the monitor's record of the old one no longer applies
    CK(cudaMemsetAsync(s->status, 0, sizeof(unsigned int), s->st));
    s->launches += 1;
    s->local = true;
    s->macro_full = false;
    s->version += 1;
    CK(cudaStreamSynchronize(s->st));
    return CLBM_OK;
}

static double from_ordered(unsigned long long v) {
    unsigned int u = (unsigned int)v;
    u = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    std::memcpy(&f, &u, 4);
    return (double)f;
}

int clbm_check(clbm_solver* s, double rho_floor, double* rho_min, double* rho_max,
               double* u_max, int64_t* nonfinite) {
    if (!s) return fail(CLBM_ERR_ARG, "clbm_check: null solver");
    if (int rc = join_bulk(s)) return rc;
    int rc = materialize(s, true);
    if (rc) return rc;
    unsigned long long h[4];
    unsigned int status = 0;
    CK(cudaMemcpyAsync(h, s->stats, sizeof(h), cudaMemcpyDeviceToHost, s->st));
    CK(cudaMemcpyAsync(&status, s->status, sizeof(status), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    if (status & kStatusWaitTimeout)
        return fail(CLBM_ERR_STATE, "clbm_check: a device wait gave up (status %u); results of "
                    "the affected steps are invalid", status);
    const bool any = h[0] != ~0ull;
    const double rmin = any ? from_ordered(h[0]) : NAN;
    const double rmax = any ? from_ordered(h[1]) : NAN;
    const double u2 = any ? from_ordered(h[2]) : NAN;
    if (rho_min) *rho_min = rmin;
    if (rho_max) *rho_max = rmax;
    if (u_max) *u_max = std::sqrt(u2);
    if (nonfinite) *nonfinite = (int64_t)h[3];
    if (h[3] > 0 || !any || rmin < rho_floor)
        return fail(CLBM_ERR_DIVERGED, "clbm_check: diverged (rho_min=%g, nonfinite=%llu)", rmin,
                    (unsigned long long)h[3]);
    if (status & kStatusDiverged)
        return fail(CLBM_ERR_DIVERGED, "clbm_check: a collision met a density below %g or not "
                    "finite since the state was last written (rho_min now %g)",
                    (double)s->c.rho_floor, rmin);
    return CLBM_OK;
}

int ibm_create(clbm_solver* s, const float* X0, const float* Y0, const float* Z0, int32_t n,
               clbm_ibm** out) {
    if (!s || !out || n < 0 || (n > 0 && (!X0 || !Y0 || !Z0)))
        return fail(CLBM_ERR_ARG, "ibm_create: invalid argument");
    *out = nullptr;
    clbm_ibm* ibm = new clbm_ibm();
    ibm->s = s;
    IbmArrays& a = ibm->a;
    a.n = n;
    a.hist_cap = kHistCap;
    auto bail = [&](int rc) { ibm_destroy(ibm); return rc; };
    if (cudaEventCreateWithFlags(&ibm->ev_box, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(CLBM_ERR_CUDA, "ibm_create: event creation failed"));
    const size_t nb = (size_t)(n > 0 ? n : 1) * sizeof(float);
    float** marr[] = {(float**)&a.X0, (float**)&a.Y0, (float**)&a.Z0, &a.X, &a.Y, &a.Z,
                      &a.VX, &a.VY, &a.Uk, &a.Vk, &a.FXk, &a.FYk};
    for (float** p : marr) {
        if (cudaMalloc(p, nb) != cudaSuccess)
            return bail(fail(CLBM_ERR_CUDA, "ibm_create: cudaMalloc failed"));
        cudaMemsetAsync(*p, 0, nb, s->st);
    }
    const size_t pb = (size_t)s->g.plane * sizeof(long long);
    if (cudaMalloc(&a.fx, pb) != cudaSuccess || cudaMalloc(&a.fy, pb) != cudaSuccess)
        return bail(fail(CLBM_ERR_CUDA, "ibm_create: cudaMalloc of force fields failed"));
    cudaMemsetAsync(a.fx, 0, pb, s->st);
    cudaMemsetAsync(a.fy, 0, pb, s->st);
    if (cudaMalloc(&a.dev, sizeof(IbmDev)) != cudaSuccess ||
        cudaMalloc(&a.hist, (size_t)kHistCap * 4 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&a.part, (size_t)kFinishBlocks * 4 * sizeof(double)) != cudaSuccess)
        return bail(fail(CLBM_ERR_CUDA, "ibm_create: cudaMalloc failed"));
    cudaMemsetAsync(a.hist, 0, (size_t)kHistCap * 4 * sizeof(double), s->st);
    IbmDev init{};
    init.step = 0;
    for (int sl = 0; sl < 2; ++sl)
        for (int e = 0; e < 6; ++e) init.box[sl][e] = kBoxEmpty;
    if (n > 0) {
        cudaMemcpyAsync((void*)a.X0, X0, n * sizeof(float), cudaMemcpyHostToDevice, s->st);
        cudaMemcpyAsync((void*)a.Y0, Y0, n * sizeof(float), cudaMemcpyHostToDevice, s->st);
        cudaMemcpyAsync((void*)a.Z0, Z0, n * sizeof(float), cudaMemcpyHostToDevice, s->st);
    }
    cudaMemcpyAsync(a.dev, &init, sizeof(init), cudaMemcpyHostToDevice, s->st);
    // Upper bound of the stencil box for any rigid motion: the template radius about the
    // pivot bounds x and y; z is fixed.
    double r2 = 0.0, zmin = 0.0, zmax = 0.0;
    for (int m = 0; m < n; ++m) {
        const double rr = (double)X0[m] * X0[m] + (double)Y0[m] * Y0[m];
        if (!std::isfinite(rr) || !std::isfinite((double)Z0[m]))
            return bail(fail(CLBM_ERR_ARG, "ibm_create: non-finite marker %d", m));
        r2 = rr > r2 ? rr : r2;
        zmin = (m == 0 || Z0[m] < zmin) ? Z0[m] : zmin;
        zmax = (m == 0 || Z0[m] > zmax) ? Z0[m] : zmax;
    }
    // marker order of the tiled spreading: Morton code of the body-frame cell (x, y, z
    // interleaved bit by bit, cells offset by 2^19), ties in marker order
    if (n > 0) {
        std::vector<unsigned long long> key(n);
        for (int m = 0; m < n; ++m) {
            const float v[3] = {X0[m], Y0[m], Z0[m]};
            unsigned long long c[3];
            for (int d = 0; d < 3; ++d) {
                const double f = std::floor((double)v[d]) + (double)(1 << 19);
                c[d] = (unsigned long long)std::min(std::max(f, 0.0), (double)((1 << 20) - 1));
            }
            unsigned long long k = 0;
            for (int b = 19; b >= 0; --b)
                for (int d = 0; d < 3; ++d) k = (k << 1) | ((c[d] >> b) & 1ull);
            key[m] = k;
        }
        std::vector<int> perm(n);
        for (int m = 0; m < n; ++m) perm[m] = m;
        std::stable_sort(perm.begin(), perm.end(), [&](int p, int q) { return key[p] < key[q]; });
        int* dperm = nullptr;
        if (cudaMalloc(&dperm, (size_t)n * sizeof(int)) != cudaSuccess)
            return bail(fail(CLBM_ERR_CUDA, "ibm_create: cudaMalloc failed"));
        a.perm = dperm;
        if (cudaMemcpy(dperm, perm.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(CLBM_ERR_CUDA, "ibm_create: marker order upload failed"));
    }
    const int span = (int)std::ceil(2.0 * std::sqrt(r2)) + 6;
    a.max_bx = std::min(s->g.nx, span);
    a.max_by = std::min(s->g.ny, span);
    a.max_bz = n > 0 ? std::min(s->g.nz, (int)(std::floor(zmax) - std::floor(zmin)) + 5) : 1;
    a.ux = s->ux;
    a.uy = s->uy;
    cudaError_t e = cudaStreamSynchronize(s->st);
    if (e != cudaSuccess) return bail(fail(CLBM_ERR_CUDA, "ibm_create: %s", cudaGetErrorString(e)));
    s->ibms.push_back(ibm);
    *out = ibm;
    return CLBM_OK;
}

int ibm_destroy(clbm_ibm* ibm) {
    if (!ibm) return CLBM_OK;
    if (clbm_solver* s = ibm->s) {
        cudaStreamSynchronize(s->st);
        if (s->g_ibm == ibm) free_graph(s);
        s->ibms.erase(std::remove(s->ibms.begin(), s->ibms.end(), ibm), s->ibms.end());
    }
    IbmArrays& a = ibm->a;
    void* ptrs[] = {(void*)a.X0, (void*)a.Y0, (void*)a.Z0, a.X, a.Y, a.Z, a.VX, a.VY, a.Uk,
                    a.Vk, a.FXk, a.FYk, a.fx, a.fy, a.dev, a.hist, a.part, (void*)a.perm};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (ibm->ev_box) cudaEventDestroy(ibm->ev_box);
    delete ibm;
    return CLBM_OK;
}

// An IBM whose solver was destroyed first stays a valid handle that can only be destroyed.
static int check_bound(const clbm_ibm* ibm, const char* fn) {
    if (!ibm) return fail(CLBM_ERR_ARG, "%s: null IBM", fn);
    if (!ibm->s) return fail(CLBM_ERR_STATE, "%s: the IBM's solver was destroyed", fn);
    return CLBM_OK;
}

int ibm_compute_force(clbm_ibm* ibm, double xc, double yc, double theta, double vx, double vy,
                      double omega) {
    if (int rc = check_bound(ibm, "ibm_compute_force")) return rc;
    MotionF mf{(float)xc, (float)yc, (float)theta, (float)vx, (float)vy, (float)omega};
    return ibm_force_impl(ibm, false, mf, clbm_motion{});
}

int ibm_compute_force_motion(clbm_ibm* ibm, const clbm_motion* m) {
    if (int rc = check_bound(ibm, "ibm_compute_force_motion")) return rc;
    if (!m) return fail(CLBM_ERR_ARG, "ibm_compute_force_motion: null motion");
    return ibm_force_impl(ibm, true, MotionF{}, *m);
}

int ibm_read_forces(const clbm_ibm* ibm, float* fx, float* fy, float* fz) {
    if (int rc = check_bound(ibm, "ibm_read_forces")) return rc;
    clbm_solver* s = ibm->s;
    if (int rc = join_bulk(s)) return rc;
    const size_t n = cells(s);
    int rc = ensure_stage(s, 2 * n * sizeof(float));
    if (rc) return rc;
    const long long* src[2] = {ibm->a.fx, ibm->a.fy};
    float* dst[2] = {fx, fy};
    for (int k = 0; k < 2; ++k) {
        if (!dst[k]) continue;
        launch_export_qfield(src[k], s->stage + k * n, s->g, 0.05f, s->st);
        CK_LAUNCH();
        s->launches += 1;
        CK(cudaMemcpyAsync(dst[k], s->stage + k * n, n * sizeof(float), cudaMemcpyDeviceToHost,
                           s->st));
    }
    CK(cudaStreamSynchronize(s->st));
    if (fz) std::memset(fz, 0, n * sizeof(float));
    return CLBM_OK;
}

int ibm_read_markers(const clbm_ibm* ibm, float* out) {
    if (int rc = check_bound(ibm, "ibm_read_markers")) return rc;
    if (!out) return fail(CLBM_ERR_ARG, "ibm_read_markers: null argument");
    const IbmArrays& a = ibm->a;
    const float* src[9] = {a.X, a.Y, a.Z, a.VX, a.VY, a.Uk, a.Vk, a.FXk, a.FYk};
    for (int k = 0; k < 9; ++k)
        if (a.n > 0)
            CK(cudaMemcpyAsync(out + (size_t)k * a.n, src[k], a.n * sizeof(float),
                               cudaMemcpyDeviceToHost, ibm->s->st));
    CK(cudaStreamSynchronize(ibm->s->st));
    return CLBM_OK;
}

int ibm_read_force_history(const clbm_ibm* ibm, int32_t count, double* out) {
    if (int rc = check_bound(ibm, "ibm_read_force_history")) return rc;
    if (!out || count < 0) return fail(CLBM_ERR_ARG, "ibm_read_force_history: bad argument");
    if (int rc = flush_sums(ibm)) return rc;
    const long long avail = std::min<long long>(ibm->calls, kHistCap);
    if (count > avail)
        return fail(CLBM_ERR_ARG, "ibm_read_force_history: %d entries requested, %lld available",
                    count, avail);
    // entries calls-count .. calls-1 occupy at most two contiguous runs of the ring
    int done = 0;
    while (done < count) {
        const long long slot = (ibm->calls - count + done) % kHistCap;
        const int run = (int)std::min<long long>(count - done, kHistCap - slot);
        CK(cudaMemcpyAsync(out + 4 * (size_t)done, ibm->a.hist + 4 * slot,
                           (size_t)run * 4 * sizeof(double), cudaMemcpyDeviceToHost, ibm->s->st));
        done += run;
    }
    CK(cudaStreamSynchronize(ibm->s->st));
    return CLBM_OK;
}

int clbm_state_bytes(const clbm_solver* s, int64_t* bytes) {
    if (!s || !bytes) return fail(CLBM_ERR_ARG, "clbm_state_bytes: null argument");
    *bytes = (int64_t)s->g.plane * (19 * (int64_t)store_bytes(s->cfg.storage) + 4 * (int64_t)sizeof(float));
    return CLBM_OK;
}

// State blob: the population buffer as stored (padded layout, storage form), then rho, ux,
// uy, uz (padded layout, float32).
int clbm_save_state(clbm_solver* s, void* out, int64_t bytes, int32_t* flags) {
    if (!s || !out || !flags) return fail(CLBM_ERR_ARG, "clbm_save_state: null argument");
    int64_t need = 0;
    clbm_state_bytes(s, &need);
    if (bytes != need)
        return fail(CLBM_ERR_ARG, "clbm_save_state: %lld bytes given, %lld needed", (long long)bytes,
                    (long long)need);
    if (int rc = join_bulk(s)) return rc;
    const size_t fb = (size_t)s->g.plane * 19 * store_bytes(s->cfg.storage);
    const size_t mb = (size_t)s->g.plane * sizeof(float);
    char* o = static_cast<char*>(out);
    CK(cudaMemcpyAsync(o, s->f[s->cur], fb, cudaMemcpyDeviceToHost, s->st));
    const float* m[4] = {s->rho, s->ux, s->uy, s->uz};
    for (int k = 0; k < 4; ++k)
        CK(cudaMemcpyAsync(o + fb + k * mb, m[k], mb, cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    *flags = (s->local ? 1 : 0) | (s->macro_full ? 2 : 0);
    return CLBM_OK;
}

int clbm_load_state(clbm_solver* s, const void* in, int64_t bytes, int32_t flags) {
    if (!s || !in) return fail(CLBM_ERR_ARG, "clbm_load_state: null argument");
    if (flags & ~3) return fail(CLBM_ERR_ARG, "clbm_load_state: unknown flags %d", flags);
    int64_t need = 0;
    clbm_state_bytes(s, &need);
    if (bytes != need)
        return fail(CLBM_ERR_ARG, "clbm_load_state: %lld bytes given, %lld needed (another lattice or "
                    "storage form)", (long long)bytes, (long long)need);
    if (int rc = join_bulk(s)) return rc;
    free_graph(s);
    const size_t fb = (size_t)s->g.plane * 19 * store_bytes(s->cfg.storage);
    const size_t mb = (size_t)s->g.plane * sizeof(float);
    const char* i = static_cast<const char*>(in);
    CK(cudaMemcpyAsync(s->f[s->cur], i, fb, cudaMemcpyHostToDevice, s->st));
    float* m[4] = {s->rho, s->ux, s->uy, s->uz};
    for (int k = 0; k < 4; ++k)
        CK(cudaMemcpyAsync(m[k], i + fb + k * mb, mb, cudaMemcpyHostToDevice, s->st));
    // a new state: the monitor's record of the old one no longer applies
    CK(cudaMemsetAsync(s->status, 0, sizeof(unsigned int), s->st));
    s->local = (flags & 1) != 0;
    s->macro_full = (flags & 2) != 0;
    s->version += 1;
    CK(cudaStreamSynchronize(s->st));
    return CLBM_OK;
}

int ibm_load_state(clbm_ibm* ibm, int64_t calls, const double* hist, int32_t count) {
    if (int rc = check_bound(ibm, "ibm_load_state")) return rc;
    if (calls < 0 || count < 0 || count > std::min<int64_t>(calls, kHistCap) || (count > 0 && !hist))
        return fail(CLBM_ERR_ARG, "ibm_load_state: bad argument");
    clbm_solver* s = ibm->s;
    if (int rc = join_bulk(s)) return rc;
    if (s->g_ibm == ibm) free_graph(s);
    IbmArrays& a = ibm->a;
    // a device record after `calls` completed calls, no force box, zero force fields (the
    // next compute_force writes them), the history ring with the given entries
    IbmDev init{};
    init.step = calls;
    init.cur = calls;
    for (int sl = 0; sl < 2; ++sl)
        for (int e = 0; e < 6; ++e) init.box[sl][e] = kBoxEmpty;
    CK(cudaMemcpyAsync(a.dev, &init, sizeof(init), cudaMemcpyHostToDevice, s->st));
    const size_t pb = (size_t)s->g.plane * sizeof(long long);
    CK(cudaMemsetAsync(a.fx, 0, pb, s->st));
    CK(cudaMemsetAsync(a.fy, 0, pb, s->st));
    CK(cudaMemsetAsync(a.hist, 0, (size_t)kHistCap * 4 * sizeof(double), s->st));
    int done = 0;
    while (done < count) {
        const long long slot = (calls - count + done) % kHistCap;
        const int run = (int)std::min<long long>(count - done, kHistCap - slot);
        CK(cudaMemcpyAsync(a.hist + 4 * slot, hist + 4 * (size_t)done, (size_t)run * 4 * sizeof(double),
                           cudaMemcpyHostToDevice, s->st));
        done += run;
    }
    CK(cudaStreamSynchronize(s->st));
    ibm->calls = calls;
    ibm->sums_pending = false;
    ibm->box_version = -1;
    return CLBM_OK;
}

int ibm_step_count(const clbm_ibm* ibm, int64_t* out) {
    if (!ibm || !out) return fail(CLBM_ERR_ARG, "ibm_step_count: null argument");
    *out = ibm->calls;
    return CLBM_OK;
}

int clbm_run(clbm_solver* s, clbm_ibm* ibm, const clbm_motion* m, int32_t nsteps,
             int32_t use_graph) {
    if (!s || nsteps < 0 || (ibm && !m)) return fail(CLBM_ERR_ARG, "clbm_run: invalid argument");
    if (ibm && ibm->s != s) return fail(CLBM_ERR_ARG, "clbm_run: IBM bound to another solver");
    int done = 0;
    const bool graph = use_graph && !s->prof;
    // Captured steps evaluate the motion law on the device (the graph replays with
    // advancing step numbers); direct launches evaluate it here in double, the arithmetic
    // of main_moving.py:65-74, and pass the float32 truncation as kernel arguments.
    bool capturing = false;
    auto one = [&]() -> int {
        if (ibm) {
            int rc;
            if (capturing) {
                rc = ibm_compute_force_motion(ibm, m);
            } else {
                const double t = (double)(ibm->calls + 1), w = m->w;
                rc = ibm_compute_force(ibm, m->x0, m->y0 + m->a_heave * std::sin(w * t),
                                       m->aoa0 + m->a_pitch * std::sin(w * t + m->phi_pitch), 0.0,
                                       m->a_heave * w * std::cos(w * t),
                                       m->a_pitch * w * std::cos(w * t + m->phi_pitch));
            }
            if (rc) return rc;
        }
        return clbm_step(s, ibm);
    };
    // steps that change the kernel variants (first pull, macro already materialised) or
    // leave an odd remainder run as plain launches
    while (done < nsteps && graph && (s->local || s->macro_full)) {
        int rc = one();
        if (rc) return rc;
        ++done;
    }
    if (graph && nsteps - done >= kGraphSteps) {
        // captured steps complete their own calls' sums; one left from before goes first
        if (ibm)
            if (int rc = flush_sums(ibm)) return rc;
        const int slot = ibm ? (int)(ibm->calls & 1) : 0;
        const bool same = s->gexec && s->g_ibm == ibm && s->g_cur == s->cur && s->g_slot == slot &&
                          (!ibm || std::memcmp(&s->g_m, m, sizeof(clbm_motion)) == 0);
        if (!same) {
            free_graph(s);
            const int cur0 = s->cur;
            const long long launches0 = s->launches;
            const long long calls0 = ibm ? ibm->calls : 0;
            if (int rc = join_bulk(s)) return rc;  // no dependency on work outside the capture
            CK(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
            capturing = true;
            int rc = CLBM_OK;
            for (int k = 0; k < kGraphSteps && !rc; ++k) rc = one();
            if (!rc) rc = join_bulk(s);  // all captured work rejoins the capture stream
            // each replay ends by copying the status word to pinned host memory, where the
            // replay loop below reads the divergence monitor without a stream sync
            if (!rc && cudaMemcpyAsync(s->h_status, s->status, sizeof(unsigned int),
                                       cudaMemcpyDeviceToHost, s->st) != cudaSuccess)
                rc = fail(CLBM_ERR_CUDA, "clbm_run: status copy could not be captured");
            capturing = false;
            cudaGraph_t graph_obj = nullptr;
            cudaError_t e = cudaStreamEndCapture(s->st, &graph_obj);
            // capture only recorded the work: restore the host mirrors
            s->cur = cur0;
            s->launches = launches0;
            if (ibm) ibm->calls = calls0;
            if (rc) {
                if (graph_obj) cudaGraphDestroy(graph_obj);
                return rc;
            }
            if (e != cudaSuccess)
                return fail(CLBM_ERR_CUDA, "clbm_run: graph capture failed: %s", cudaGetErrorString(e));
            // keep the stream priorities of the captured kernels (IBM chain over bulk pass)
            e = cudaGraphInstantiateWithFlags(&s->gexec, graph_obj, cudaGraphInstantiateFlagUseNodePriority);
            cudaGraphDestroy(graph_obj);
            if (e != cudaSuccess)
                return fail(CLBM_ERR_CUDA, "clbm_run: graph instantiate failed: %s", cudaGetErrorString(e));
            s->g_ibm = ibm;
            if (ibm) s->g_m = *m;
            s->g_cur = cur0;
            s->g_slot = slot;
        }
        const int per = ibm ? (ibm->a.n > 0 ? kKernelsPerIbmStep : kKernelsPerIbmStep - 2) : 1;
        // a direct step before the replay may have left its bulk pass running on the second
        // stream; the graph's first kernels read the state that pass writes
        if (int rc = join_bulk(s)) return rc;
        // At most kReplaysInFlight replays are queued: before each launch beyond that, wait
        // for the oldest and read the status word it copied out. A run that diverged stops
        // within kReplaysInFlight + 1 replays of the step that diverged (main_moving.py:143-145
        // breaks its loop on the same condition at its vis steps).
        *s->h_status = 0;
        long long replays = 0;
        while (nsteps - done >= kGraphSteps) {
            if (replays >= kReplaysInFlight) {
                CK(cudaEventSynchronize(s->ev_replay[replays % kReplaysInFlight]));
                const unsigned int st_word = *(volatile unsigned int*)s->h_status;
                if (st_word & (kStatusDiverged | kStatusWaitTimeout | kStatusBounds)) {
                    s->local = false;
                    s->macro_full = false;
                    if (st_word & kStatusWaitTimeout)
                        return fail(CLBM_ERR_STATE, "clbm_run: a device wait gave up (status %u)",
                                    st_word);
                    if (st_word & kStatusBounds)
                        return fail(CLBM_ERR_STATE, "clbm_run: an access outside its array was "
                                    "caught and skipped (bounds-checked build, status %u)", st_word);
                    return fail(CLBM_ERR_DIVERGED, "clbm_run: diverged: a collision met a "
                                "density below %g or not finite; stopped after %d of %d steps",
                                (double)s->c.rho_floor, done, nsteps);
                }
            }
            CK(cudaGraphLaunch(s->gexec, s->st));
            CK(cudaEventRecord(s->ev_replay[replays % kReplaysInFlight], s->st));
            ++replays;
            done += kGraphSteps;
            s->version += kGraphSteps;
            s->launches += kGraphSteps * per;
            if (ibm) ibm->calls += kGraphSteps;
        }
        s->local = false;
        s->macro_full = false;
    }
    while (done < nsteps) {
        int rc = one();
        if (rc) return rc;
        ++done;
    }
    return join_bulk(s);  // the run's work is complete on the solver stream
}

int clbm_synchronize(clbm_solver* s) {
    if (!s) return fail(CLBM_ERR_ARG, "clbm_synchronize: null solver");
    if (int rc = join_bulk(s)) return rc;
    unsigned int status = 0;
    CK(cudaMemcpyAsync(&status, s->status, sizeof(status), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    if (status & kStatusWaitTimeout)
        return fail(CLBM_ERR_STATE, "clbm_synchronize: a device wait gave up (status %u)", status);
    if (status & kStatusBounds)
        return fail(CLBM_ERR_STATE, "clbm_synchronize: an access outside its array was caught and "
                    "skipped (bounds-checked build, status %u)", status);
    if (status & kStatusDiverged)
        return fail(CLBM_ERR_DIVERGED, "clbm_synchronize: diverged: a collision met a density "
                    "below %g or not finite", (double)s->c.rho_floor);
    return CLBM_OK;
}

int clbm_bounds_checked(int32_t* on) {
    if (!on) return fail(CLBM_ERR_ARG, "clbm_bounds_checked: null argument");
    *on = kBoundsChecked ? 1 : 0;
    return CLBM_OK;
}

int clbm_selftest_bounds(clbm_solver* s) {
    if (!s) return fail(CLBM_ERR_ARG, "clbm_selftest_bounds: null solver");
    if (!kBoundsChecked) return fail(CLBM_ERR_STATE, "clbm_selftest_bounds: not the bounds-checked build");
    if (int rc = join_bulk(s)) return rc;
    CK(cudaStreamSynchronize(s->st));
    launch_bounds_selftest(s->g, s->st);
    CK_LAUNCH();
    s->launches += 1;
    unsigned int status = 0;
    CK(cudaMemcpyAsync(&status, s->status, sizeof(status), cudaMemcpyDeviceToHost, s->st));
    CK(cudaMemsetAsync(s->status, 0, sizeof(unsigned int), s->st));
    CK(cudaStreamSynchronize(s->st));
    if (status & kStatusBounds)
        return fail(CLBM_ERR_STATE, "clbm_selftest_bounds: the index test past the end was reported "
                    "as intended (status %u)", status);
    return fail(CLBM_ERR_CUDA, "clbm_selftest_bounds: the index test was not reported");
}

int clbm_selftest_wait_timeout(clbm_solver* s, int32_t spin_limit) {
    // at least 1024 polls, so every block's copies have landed before it gives up and exits
    if (!s || spin_limit < 1024)
        return fail(CLBM_ERR_ARG, "clbm_selftest_wait_timeout: spin_limit must be >= 1024");
    if (int rc = join_bulk(s)) return rc;
    CK(cudaStreamSynchronize(s->st));
    Grid g = s->g;
    g.spin_limit = spin_limit;
    g.extra_tx = 16;  // one more 16-byte chunk than is ever copied: every wait runs out
    ForceArgs fa{};
    launch_stream_collide(s->cfg.storage, !s->local, kForceNone, kVariantStaged, s->f[s->cur],
                          s->f[1 - s->cur], g, s->c, fa, s->st);
    CK_LAUNCH();
    s->launches += 1;
    unsigned int status = 0;
    CK(cudaMemcpyAsync(&status, s->status, sizeof(status), cudaMemcpyDeviceToHost, s->st));
    CK(cudaMemsetAsync(s->status, 0, sizeof(unsigned int), s->st));
    CK(cudaStreamSynchronize(s->st));
    if (status)
        return fail(CLBM_ERR_STATE, "clbm_selftest_wait_timeout: bounded wait gave up as intended "
                    "(status %u)", status);
    return fail(CLBM_ERR_CUDA, "clbm_selftest_wait_timeout: the wait did not report a timeout");
}

int clbm_stream(const clbm_solver* s, void** out) {
    if (!s || !out) return fail(CLBM_ERR_ARG, "clbm_stream: null argument");
    // work queued so far is complete on the returned stream
    if (int rc = join_bulk(const_cast<clbm_solver*>(s))) return rc;
    *out = (void*)s->st;
    return CLBM_OK;
}

int clbm_profile_enable(clbm_solver* s, int32_t on) {
    if (!s) return fail(CLBM_ERR_ARG, "clbm_profile_enable: null solver");
    CK(cudaStreamSynchronize(s->st));
    s->prof = on != 0;
    s->ev_used = 0;
    return CLBM_OK;
}

int clbm_profile_read(clbm_solver* s, double* fused_ms, int64_t* fused_launches,
                      int64_t* total_launches) {
    if (!s) return fail(CLBM_ERR_ARG, "clbm_profile_read: null solver");
    if (int rc = join_bulk(s)) return rc;
    CK(cudaStreamSynchronize(s->st));
    double ms = 0.0;
    for (size_t i = 0; i + 1 < s->ev_used; i += 2) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, s->ev[i], s->ev[i + 1]));
        ms += t;
    }
    if (fused_ms) *fused_ms = ms;
    if (fused_launches) *fused_launches = (int64_t)(s->ev_used / 2);
    if (total_launches) *total_launches = s->launches;
    return CLBM_OK;
}

int clbm_profile_read_split(clbm_solver* s, double* bulk_ms, int64_t* bulk_launches,
                            double* box_ms, int64_t* box_launches) {
    if (!s) return fail(CLBM_ERR_ARG, "clbm_profile_read_split: null solver");
    if (int rc = join_bulk(s)) return rc;
    CK(cudaStreamSynchronize(s->st));
    double ms[2] = {0.0, 0.0};
    int64_t n[2] = {0, 0};
    for (size_t i = 0; i + 1 < s->ev_used; i += 2) {
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, s->ev[i], s->ev[i + 1]));
        const int tag = (i / 2 < s->ev_tag.size()) ? s->ev_tag[i / 2] : 0;
        ms[tag] += t;
        n[tag] += 1;
    }
    if (bulk_ms) *bulk_ms = ms[0];
    if (bulk_launches) *bulk_launches = n[0];
    if (box_ms) *box_ms = ms[1];
    if (box_launches) *box_launches = n[1];
    return CLBM_OK;
}

int clbm_device_bytes(const clbm_solver* s, int64_t* out) {
    if (!s || !out) return fail(CLBM_ERR_ARG, "clbm_device_bytes: null argument");
    const size_t pb = (size_t)s->g.plane * sizeof(float);
    size_t b = 2 * (size_t)s->g.plane * 19 * store_bytes(s->cfg.storage) + 4 * pb;
    if (s->dfx) b += 3 * pb;
    b += s->stage_bytes;
    *out = (int64_t)b;
    return CLBM_OK;
}

int clbm_closure_set(clbm_solver* s, const float* params) {
    if (!s) return fail(CLBM_ERR_ARG, "clbm_closure_set: null solver");
    if (int rc = join_bulk(s)) return rc;
    CK(cudaStreamSynchronize(s->st));
    CK(cudaStreamSynchronize(s->st2));
    free_graph(s);  // the captured bulk-pass kernel changes
    if (!params) {
        s->closure = false;
        return CLBM_OK;
    }
    for (int i = 0; i < closure::kParams; ++i)
        if (!std::isfinite(params[i])) return fail(CLBM_ERR_ARG, "clbm_closure_set: parameter %d not finite", i);
    if (!s->cl_params) CK(cudaMalloc(&s->cl_params, sizeof(float) * closure::kParams));
    if (!s->cl_img) CK(cudaMalloc(&s->cl_img, sizeof(uint16_t) * closure::kImgElems));
    CK(cudaMemcpyAsync(s->cl_params, params, sizeof(float) * closure::kParams, cudaMemcpyHostToDevice, s->st));
    launch_closure_images(s->cl_params, s->cl_img, s->st);
    CK_LAUNCH();
    CK(cudaStreamSynchronize(s->st));
    s->cl_grid = closure_grid(s->cfg.storage);
    s->closure = true;
    s->launches += 1;
    return CLBM_OK;
}

int clbm_binary_version(int32_t* binary, int32_t* ptx) {
    if (!binary || !ptx) return fail(CLBM_ERR_ARG, "clbm_binary_version: null argument");
    int b = 0, p = 0;
    const cudaError_t err = stream_collide_binary_version(&b, &p);
    if (err != cudaSuccess) return fail(CLBM_ERR_CUDA, "clbm_binary_version: %s", cudaGetErrorString(err));
    *binary = b;
    *ptx = p;
    return CLBM_OK;
}

int clbm_kernel_variant(const clbm_solver* s, int32_t* variant, float* ms_per_launch) {
    if (!s || !variant) return fail(CLBM_ERR_ARG, "clbm_kernel_variant: invalid argument");
    *variant = s->variant;
    if (ms_per_launch)
        for (int v = 0; v < kVariants; ++v) ms_per_launch[v] = s->variant_ms[v];
    return CLBM_OK;
}

int clbm_set_rho_floor(clbm_solver* s, double rho_floor) {
    if (!s || std::isnan(rho_floor)) return fail(CLBM_ERR_ARG, "clbm_set_rho_floor: invalid argument");
    if (int rc = join_bulk(s)) return rc;
    CK(cudaStreamSynchronize(s->st));
    s->c.rho_floor = rho_floor < 0.0 ? -3.0e38f : (float)rho_floor;
    free_graph(s);  // captured launches hold the old coefficients
    return CLBM_OK;
}

int clbm_host_alloc(int64_t bytes, void** out) {
    if (!out || bytes <= 0) return fail(CLBM_ERR_ARG, "clbm_host_alloc: invalid argument");
    CK(cudaHostAlloc(out, (size_t)bytes, cudaHostAllocDefault));
    return CLBM_OK;
}

int clbm_host_free(void* p) {
    if (p) CK(cudaFreeHost(p));
    return CLBM_OK;
}

}  // extern "C"

// ====================================================================== ensemble
struct clbm_ensemble {
    std::vector<clbm_solver*> s;
    std::vector<clbm_ibm*> ibm;
    std::vector<clbm_motion> m;
    int n = 0;
    int storage = 0;
    EnsDesc* d_desc = nullptr;
    long long* d_tile0 = nullptr;
    long long* d_off = nullptr;  // flat force-box offsets: new box [n + 1], then previous box [n + 1]
    int flat_grid = 0;           // blocks of the flat band-prepare and box passes
    long long ntiles = 0;
    int bx = 128;            // bulk tile width (cells)
    int grid = 0;            // persistent bulk blocks
    // instances grouped by row width, whole rows per block (rows = true when the autotuner
    // chose it), rows_per_tile rows per tile
    struct Group {
        EnsDesc* d = nullptr;
        long long* tile0 = nullptr;
        int n = 0;
        long long ntiles = 0;
        int threads = 0;
        bool idx32 = true;   // 19 * plane of every member below 2^32
    };
    std::vector<Group> groups;
    bool rows = false;
    int rows_per_tile = 1;
    // streams of the groups after the first (the groups' bulk launches run concurrently, so
    // the short launches of the small groups fill each other's ramp-up and tail)
    std::vector<cudaStream_t> gst;
    std::vector<cudaEvent_t> gev;   // [0]: fork; [1 + k]: end of group k + 1
    // bulk pass as one single-lattice stream-collide launch per member (members = true when
    // the autotuner chose it): members in order of size, round-robin over kMemberStreams
    // concurrent streams
    bool members = false;
    std::vector<int> morder;
    std::vector<cudaStream_t> mst;
    std::vector<cudaEvent_t> mev;   // [0]: fork; [1 + k]: end of stream k
    float bulk_ms = 0.f;     // time of one bulk pass of the chosen schedule at creation
    int max_marker_blocks = 0, max_spread_blocks = 0;
    int cur = 0;
    bool local = true, macro_full = true;
    cudaStream_t st = nullptr, st2 = nullptr;
    cudaEvent_t ev_box = nullptr, ev_bulk = nullptr, ev_sync = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int g_cur = -1;
    long long launches = 0;
    // the whole step as one persistent cooperative launch (CLBM_ENS_STEP=persistent at
    // creation): EnsPersArgs template, grid, and its device arrays
    bool pers = false;
    bool pers_idx32 = true;
    int pers_grid = 0;
    long long* d_pers = nullptr;   // mk0, sw0, off_rows: [n + 1] each
    std::unique_ptr<EnsPersTable> ptab;   // parameter table of the bulk tiles
    unsigned* d_bar = nullptr;     // grid barrier: arrivals, generation, error bits
    IbmDev* d_nodev = nullptr;     // zeroed (empty force band)
    unsigned long long* d_stamps = nullptr;   // phase clock of the last persistent step
    EnsPersArgs pa{};
};

namespace {

// Descriptor of member i (tile0 left to the caller).
EnsDesc member_desc(const clbm_ensemble* e, int i) {
    const clbm_solver* s = e->s[i];
    EnsDesc D{};
    D.g = s->g;
    D.c = s->c;
    D.f[0] = s->f[0];
    D.f[1] = s->f[1];
    D.rho = s->rho; D.ux = s->ux; D.uy = s->uy; D.uz = s->uz;
    D.has_ibm = e->ibm[i] != nullptr;
    if (D.has_ibm) D.a = e->ibm[i]->a;
    D.m = e->m[i];
    D.cells = s->g.nx * s->g.ny * s->g.nz;
    return D;
}

void ens_free_groups(clbm_ensemble* e) {
    for (auto& G : e->groups) {
        if (G.d) cudaFree(G.d);
        if (G.tile0) cudaFree(G.tile0);
    }
    e->groups.clear();
}

// Members grouped by the threads a whole row needs (a multiple of 32; two cells per thread
// in the 16-bit forms, one in float32; rows up to 512 cells); each group's descriptors list
// its members with tiles of R rows. No groups when a row is wider.
int ens_groups(clbm_ensemble* e, int R) {
    ens_free_groups(e);
    e->rows_per_tile = R;
    const bool f32 = e->storage == CLBM_STORE_F32;   // one cell per thread, rows up to 512
    std::vector<int> th(e->n);
    for (int i = 0; i < e->n; ++i) {
        const int nx = e->s[i]->g.nx;
        if (nx > 512) return CLBM_OK;
        th[i] = f32 ? (nx + 31) / 32 * 32 : (nx + 63) / 64 * 32;
    }
    std::vector<int> widths(th);
    std::sort(widths.begin(), widths.end());
    widths.erase(std::unique(widths.begin(), widths.end()), widths.end());
    for (int w : widths) {
        std::vector<EnsDesc> h;
        std::vector<long long> t0;
        long long tiles = 0;
        bool idx32 = true;
        for (int i = 0; i < e->n; ++i) {
            if (th[i] != w) continue;
            EnsDesc D = member_desc(e, i);
            D.tile0 = tiles;
            t0.push_back(tiles);
            tiles += ((long long)D.g.ny * D.g.nz + R - 1) / R;
            idx32 = idx32 && 19LL * D.g.plane <= 0xffffffffLL;
            h.push_back(D);
        }
        clbm_ensemble::Group gr;
        gr.n = (int)h.size();
        gr.ntiles = tiles;
        gr.threads = w;
        gr.idx32 = idx32;
        e->groups.push_back(gr);
        clbm_ensemble::Group& G = e->groups.back();
        CK(cudaMalloc(&G.d, sizeof(EnsDesc) * G.n));
        CK(cudaMalloc(&G.tile0, sizeof(long long) * G.n));
        CK(cudaMemcpyAsync(G.d, h.data(), sizeof(EnsDesc) * G.n, cudaMemcpyHostToDevice, e->st));
        CK(cudaMemcpyAsync(G.tile0, t0.data(), sizeof(long long) * G.n, cudaMemcpyHostToDevice, e->st));
    }
    // the group with the most tiles first
    std::stable_sort(e->groups.begin(), e->groups.end(),
                     [](const clbm_ensemble::Group& a, const clbm_ensemble::Group& b) { return a.ntiles > b.ntiles; });
    int lo = 0, hi = 0;
    CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    while (e->gst.size() + 1 < e->groups.size()) {
        cudaStream_t st;
        CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, lo));
        e->gst.push_back(st);
    }
    while (e->gev.size() < e->groups.size()) {
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        e->gev.push_back(ev);
    }
    CK(cudaStreamSynchronize(e->st));
    return CLBM_OK;
}

// Bulk pass in the row mode: one launch per group, the first on `st`, the others on their
// own streams forked from and joined back to `st`.
int ens_bulk_rows(clbm_ensemble* e, bool pull, cudaStream_t st) {
    const size_t ng = e->groups.size();
    if (ng > 1) CK(cudaEventRecord(e->gev[0], st));
    for (size_t k = 0; k < ng; ++k) {
        const auto& G = e->groups[k];
        cudaStream_t sk = k == 0 ? st : e->gst[k - 1];
        if (k > 0) CK(cudaStreamWaitEvent(sk, e->gev[0], 0));
        launch_ens_bulk_rows(e->storage, pull, G.threads, e->rows_per_tile, G.idx32, G.d, G.tile0, G.n,
                             G.ntiles, e->cur, (int)std::min<long long>(G.ntiles, 1LL << 30), sk);
        if (k > 0) CK(cudaEventRecord(e->gev[k], sk));
    }
    for (size_t k = 1; k < ng; ++k) CK(cudaStreamWaitEvent(st, e->gev[k], 0));
    return CLBM_OK;
}

constexpr int kMemberStreams = 8;

// Streams and order of the per-member bulk launches.
int ens_members_setup(clbm_ensemble* e) {
    if (!e->mst.empty()) return CLBM_OK;
    int lo = 0, hi = 0;
    CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    const int k = std::max(1, std::min(knob("CLBM_ENS_MEMBER_STREAMS", kMemberStreams), e->n));
    for (int i = 0; i < k; ++i) {
        cudaStream_t st;
        CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, lo));
        e->mst.push_back(st);
    }
    for (int i = 0; i <= k; ++i) {
        cudaEvent_t ev;
        CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        e->mev.push_back(ev);
    }
    e->morder.resize(e->n);
    for (int i = 0; i < e->n; ++i) e->morder[i] = i;
    std::stable_sort(e->morder.begin(), e->morder.end(), [&](int a, int b) {
        return (long long)e->s[a]->g.nx * e->s[a]->g.ny * e->s[a]->g.nz >
               (long long)e->s[b]->g.nx * e->s[b]->g.ny * e->s[b]->g.nz;
    });
    return CLBM_OK;
}

// The bulk pass as one launch of the single-lattice stream-collide kernel per member (the
// one-cell kernel in float32, the two-cell kernel in the 16-bit forms), skipping the
// member's force box, forked from st over the member streams and joined back into it.
int ens_bulk_members(clbm_ensemble* e, bool pull, cudaStream_t st) {
    const int k = (int)e->mst.size();
    CK(cudaEventRecord(e->mev[0], st));
    for (int j = 0; j < k; ++j) CK(cudaStreamWaitEvent(e->mst[j], e->mev[0], 0));
    const int variant = e->storage == CLBM_STORE_F32 ? kVariantCell : kVariantPair;
    for (int r = 0; r < e->n; ++r) {
        const int i = e->morder[r];
        const clbm_solver* s = e->s[i];
        const clbm_ibm* b = e->ibm[i];
        ForceArgs fa{};
        int fmode = kForceNone;
        if (b) {
            fa.dev = b->a.dev;
            fa.slot = -1;   // the member's current call, read on the device
            fmode = kForceSkipBand;
        }
        launch_stream_collide(e->storage, pull, fmode, variant, s->f[e->cur], s->f[e->cur ^ 1], s->g,
                              s->c, fa, e->mst[r % k]);
    }
    for (int j = 0; j < k; ++j) {
        CK(cudaEventRecord(e->mev[1 + j], e->mst[j]));
        CK(cudaStreamWaitEvent(st, e->mev[1 + j], 0));
    }
    return CLBM_OK;
}

// Device descriptors for tile width bx; returns the number of bulk tiles.
int ens_upload(clbm_ensemble* e, int bx) {
    std::vector<EnsDesc> h(e->n);
    std::vector<long long> t0(e->n);
    long long tiles = 0;
    for (int i = 0; i < e->n; ++i) {
        clbm_solver* s = e->s[i];
        EnsDesc& D = h[i];
        D = member_desc(e, i);
        D.tile0 = tiles;
        t0[i] = tiles;
        // a tile is a run of bx consecutive cells (float32) or a segment of bx cells of one
        // row (16-bit forms: the two cells of a thread and a warp's rows stay in one row)
        if (e->storage != CLBM_STORE_F32)
            tiles += (long long)((s->g.nx + bx - 1) / bx) * s->g.ny * s->g.nz;
        else
            tiles += (D.cells + bx - 1) / bx;
    }
    CK(cudaMemcpyAsync(e->d_desc, h.data(), sizeof(EnsDesc) * e->n, cudaMemcpyHostToDevice, e->st));
    CK(cudaMemcpyAsync(e->d_tile0, t0.data(), sizeof(long long) * e->n, cudaMemcpyHostToDevice, e->st));
    CK(cudaStreamSynchronize(e->st));
    e->ntiles = tiles;
    e->bx = bx;
    return CLBM_OK;
}

// The ensemble's bulk-pass schedule: tile width 128 or 256 cells, and persistent blocks
// (4 or 8 per SM) or one block per tile; each candidate is timed over three launches.
int ens_tune(clbm_ensemble* e) {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_bx = 128, best_grid = 4 * sms;
    for (int bx : {128, 256}) {
        if (int rc = ens_upload(e, bx)) return rc;
        for (int per_sm : {4, 8, 0}) {
            const long long g = per_sm ? (long long)per_sm * sms : e->ntiles;
            const int grid = (int)std::min<long long>(g, 1LL << 30);
            launch_ens_bulk(e->storage, true, bx, e->d_desc, e->d_tile0, e->n, e->ntiles, e->cur,
                            grid, e->st);
            CK(cudaEventRecord(e0, e->st));
            for (int k = 0; k < 3; ++k)
                launch_ens_bulk(e->storage, true, bx, e->d_desc, e->d_tile0, e->n, e->ntiles,
                                e->cur, grid, e->st);
            CK(cudaEventRecord(e1, e->st));
            CK(cudaEventSynchronize(e1));
            CK_LAUNCH();
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, e0, e1));
            e->launches += 4;
            if (ms < best) {
                best = ms;
                best_bx = bx;
                best_grid = grid;
            }
        }
    }
    e->grid = best_grid;
    e->bulk_ms = best / 3.0f;
    e->rows = false;
    // whole rows per block, instances grouped by row width, R rows per tile (the instance
    // lookup is paid once per tile); CLBM_ENS_ROWS=1 / 0 forces / forbids the row mode
    // (tests), CLBM_ENS_ROWS_R fixes R; default: the fastest
    const int force = knob("CLBM_ENS_ROWS", -1);
    const int fixed_r = knob("CLBM_ENS_ROWS_R", 0);
    float best_rows = 1e30f;
    int best_r = 1;
    const std::vector<int> cand_r = fixed_r > 0 ? std::vector<int>{fixed_r} : std::vector<int>{1, 2, 4, 8};
    for (int R : cand_r) {
        if (int rc = ens_groups(e, R)) return rc;
        if (e->groups.empty()) break;
        if (int rc = ens_bulk_rows(e, true, e->st)) return rc;
        CK(cudaEventRecord(e0, e->st));
        for (int k = 0; k < 3; ++k)
            if (int rc = ens_bulk_rows(e, true, e->st)) return rc;
        CK(cudaEventRecord(e1, e->st));
        CK(cudaEventSynchronize(e1));
        CK_LAUNCH();
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        e->launches += 4 * (long long)e->groups.size();
        if (ms < best_rows) {
            best_rows = ms;
            best_r = R;
        }
    }
    if (!e->groups.empty() && (force == 1 || (force != 0 && best_rows < best))) {
        if (int rc = ens_groups(e, best_r)) return rc;
        e->rows = true;
        e->bulk_ms = best_rows / 3.0f;
    }
    // one single-lattice launch per member over concurrent streams; CLBM_ENS_MEMBERS=1 / 0
    // forces / forbids it (tests), otherwise kept when faster than the schedule above
    const int force_m = knob("CLBM_ENS_MEMBERS", -1);
    if (force_m != 0 && force != 1) {
        if (int rc = ens_members_setup(e)) return rc;
        if (int rc = ens_bulk_members(e, true, e->st)) return rc;
        CK(cudaEventRecord(e0, e->st));
        for (int k = 0; k < 3; ++k)
            if (int rc = ens_bulk_members(e, true, e->st)) return rc;
        CK(cudaEventRecord(e1, e->st));
        CK(cudaEventSynchronize(e1));
        CK_LAUNCH();
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        e->launches += 4LL * e->n;
        if (force_m == 1 || ms / 3.0f < e->bulk_ms) {
            e->members = true;
            e->rows = false;
            e->bulk_ms = ms / 3.0f;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ens_upload(e, best_bx);
}

// Set up the persistent step: per-member offsets of the virtual marker blocks and
// spreading warps, the parameter table of the bulk tiles (members' constants and first
// block tiles), the share of the bulk pass done in each phase (CLBM_ENS_PERS_SPLIT="a,b,c":
// the cumulative fractions done by the ends of phases 2, 3 and 4; default 0.1,0.3,0.7)
// and the grid: every block resident (the cooperative launch refuses a larger grid).
int ens_pers_setup(clbm_ensemble* e) {
    const int n = e->n;
    if (n > kPersMaxMembers)
        return fail(CLBM_ERR_ARG, "clbm_ensemble_create: the persistent step takes at most %d members",
                    kPersMaxMembers);
    std::vector<long long> h(3 * (size_t)(n + 1), 0);
    long long* mk0 = h.data();
    long long* sw0 = mk0 + n + 1;
    e->ptab.reset(new EnsPersTable());
    EnsPersTable& tb = *e->ptab;
    CK(cudaMalloc(&e->d_nodev, sizeof(IbmDev)));
    CK(cudaMemsetAsync(e->d_nodev, 0, sizeof(IbmDev), e->st));
    bool idx32 = true;
    long long bt = 0;
    for (int i = 0; i < n; ++i) {
        const clbm_solver* s = e->s[i];
        const clbm_ibm* b = e->ibm[i];
        const long long nm = b ? b->a.n : 0;
        mk0[i + 1] = mk0[i] + (nm + kEnsMarkerBlock - 1) / kEnsMarkerBlock;
        sw0[i + 1] = sw0[i] + (nm + kSpreadMarkersPerWarp - 1) / kSpreadMarkersPerWarp;
        const EnsDesc D = member_desc(e, i);
        const long long cells = (long long)s->g.nx * s->g.ny * s->g.nz;
        const long long wt = e->storage == CLBM_STORE_F32 ? (cells + 31) / 32
                                                         : (long long)((s->g.nx + 63) / 64) * s->g.ny * s->g.nz;
        EnsMember& M = tb.m[i];
        M.g = D.g;
        M.c = D.c;
        M.f[0] = D.f[0];
        M.f[1] = D.f[1];
        M.dev = D.has_ibm ? D.a.dev : e->d_nodev;
        M.cells = D.cells;
        M.wtiles = (int)wt;
        tb.bt0[i] = (int)bt;
        bt += (wt + kPersTileWarps - 1) / kPersTileWarps;
        idx32 = idx32 && 19LL * s->g.plane <= 0xffffffffLL;
    }
    if (bt >= (1LL << 30))
        return fail(CLBM_ERR_ARG, "clbm_ensemble_create: too many cells for the persistent step");
    tb.bt0[n] = (int)bt;
    double f[3] = {0.1, 0.3, 0.7};
    if (const char* env = std::getenv("CLBM_ENS_PERS_SPLIT")) {
        double a = 0, b = 0, c = 0;
        if (std::sscanf(env, "%lf,%lf,%lf", &a, &b, &c) == 3 && 0 <= a && a <= b && b <= c && c <= 1) {
            f[0] = a; f[1] = b; f[2] = c;
        }
    }
    EnsPersArgs& p = e->pa;
    p.bt_split[0] = 0;
    for (int k = 0; k < 3; ++k) p.bt_split[k + 1] = (int)(f[k] * (double)bt);
    p.bt_split[4] = (int)bt;
    p.mk_total = mk0[n];
    p.sw_total = sw0[n];
    p.n = n;
    p.fin_blocks = kFinishBlocks / 4;   // 256-thread blocks: the threads of 64 of 64
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int per_sm = ens_persistent_blocks_per_sm(e->storage, idx32);
    if (per_sm < 1 || sms < 1)
        return fail(CLBM_ERR_CUDA, "clbm_ensemble_create: no resident block for the persistent step");
    CK(cudaMalloc(&e->d_pers, sizeof(long long) * h.size()));
    CK(cudaMalloc(&e->d_bar, 4 * sizeof(unsigned)));
    CK(cudaMalloc(&e->d_stamps, 6 * sizeof(unsigned long long)));
    CK(cudaMemsetAsync(e->d_stamps, 0, 6 * sizeof(unsigned long long), e->st));
    CK(cudaMemcpyAsync(e->d_pers, h.data(), sizeof(long long) * h.size(), cudaMemcpyHostToDevice, e->st));
    CK(cudaMemsetAsync(e->d_bar, 0, 4 * sizeof(unsigned), e->st));
    CK(cudaStreamSynchronize(e->st));
    p.mk0 = e->d_pers;
    p.sw0 = e->d_pers + n + 1;
    p.off_rows = e->d_pers + 2 * (n + 1);
    p.off_new = e->d_off;
    p.off_old = e->d_off + n + 1;
    p.bar = e->d_bar;
    p.nodev = e->d_nodev;
    p.stamps = e->d_stamps;
    e->pers_idx32 = idx32;
    e->pers_grid = per_sm * sms;
    e->pers = true;
    return CLBM_OK;
}

// Error bits of the persistent step's barrier (a wait ran out): reported once, then
// cleared.
int ens_pers_check(clbm_ensemble* e, const char* who) {
    if (!e->pers) return CLBM_OK;
    unsigned err = 0;
    CK(cudaMemcpyAsync(&err, e->d_bar + 2, sizeof(err), cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
    if (!err) return CLBM_OK;
    CK(cudaMemsetAsync(e->d_bar, 0, 4 * sizeof(unsigned), e->st));
    CK(cudaStreamSynchronize(e->st));
    return fail(CLBM_ERR_STATE, "%s: a grid-barrier wait of the persistent step ran out "
                "(bits %u); the members' state is not valid", who, err);
}

// Kernel launches of one ensemble step: the six of the IBM chain and the box pass, and the
// bulk pass's (one, one per row-width group, or one per member); one for the persistent step.
long long ens_step_launches(const clbm_ensemble* e) {
    if (e->pers) return 1;
    return 6 + (e->members ? e->n : e->rows ? (long long)e->groups.size() : 1);
}

int ens_step(clbm_ensemble* e) {
    const bool pull = !e->local;
    if (e->pers) {
        EnsPersArgs p = e->pa;
        p.parity = e->cur;
        p.compute_macro = !e->macro_full;
        const cudaError_t err = launch_ens_persistent(e->storage, pull, e->pers_idx32, e->d_desc, p,
                                                      *e->ptab, e->pers_grid, e->st);
        if (err != cudaSuccess)
            return fail(CLBM_ERR_CUDA, "ensemble persistent step: %s", cudaGetErrorString(err));
        e->launches += 1;
        e->cur ^= 1;
        e->local = false;
        e->macro_full = false;
        return CLBM_OK;
    }
    launch_ens_markers(e->d_desc, e->n, e->max_marker_blocks, e->st);
    CK(cudaEventRecord(e->ev_box, e->st));
    long long* off_new = e->d_off;
    long long* off_old = e->d_off + e->n + 1;
    launch_ens_box_scan(e->d_desc, e->n, off_new, off_old, e->st);
    launch_ens_band_prepare_flat(e->storage, pull, e->d_desc, e->n, off_new, off_old, e->cur, !e->macro_full,
                                 e->flat_grid, e->st);
    launch_ens_interp_spread(e->d_desc, e->n, e->max_spread_blocks, e->st);
    launch_ens_finish(e->d_desc, e->n, e->st);
    CK(cudaStreamWaitEvent(e->st2, e->ev_box, 0));
    if (e->members) {
        if (int rc = ens_bulk_members(e, pull, e->st2)) return rc;
    } else if (e->rows) {
        if (int rc = ens_bulk_rows(e, pull, e->st2)) return rc;
    } else launch_ens_bulk(e->storage, pull, e->bx, e->d_desc, e->d_tile0, e->n, e->ntiles, e->cur,
                         e->grid, e->st2);
    CK(cudaEventRecord(e->ev_bulk, e->st2));
    launch_ens_box_flat(e->storage, pull, e->d_desc, e->n, off_new, e->cur, e->flat_grid, e->st);
    CK(cudaStreamWaitEvent(e->st, e->ev_bulk, 0));
    CK_LAUNCH();
    e->launches += ens_step_launches(e);
    e->cur ^= 1;
    e->local = false;
    e->macro_full = false;
    return CLBM_OK;
}

void ens_free_graph(clbm_ensemble* e) {
    if (e->gexec) cudaGraphExecDestroy(e->gexec);
    e->gexec = nullptr;
    e->g_cur = -1;
}

}  // namespace

extern "C" {

int clbm_ensemble_create(clbm_solver* const* solvers, clbm_ibm* const* ibms,
                         const clbm_motion* motions, int32_t n, clbm_ensemble** out) {
    if (!solvers || !motions || !out || n < 1 || n > 4096)
        return fail(CLBM_ERR_ARG, "clbm_ensemble_create: invalid argument");
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        clbm_solver* s = solvers[i];
        if (!s) return fail(CLBM_ERR_ARG, "clbm_ensemble_create: null solver %d", i);
        if ((long long)s->g.nx * s->g.ny * s->g.nz > (1LL << 30))
            return fail(CLBM_ERR_ARG, "clbm_ensemble_create: member %d has more than 2^30 cells", i);
        if (s->cfg.storage != solvers[0]->cfg.storage || s->cfg.device != solvers[0]->cfg.device)
            return fail(CLBM_ERR_ARG, "clbm_ensemble_create: solvers differ in storage or device");
        if (s->cur != solvers[0]->cur || s->local != solvers[0]->local ||
            s->macro_full != solvers[0]->macro_full)
            return fail(CLBM_ERR_STATE, "clbm_ensemble_create: solvers are not at the same step");
        if (ibms && ibms[i] && ibms[i]->s != s)
            return fail(CLBM_ERR_ARG, "clbm_ensemble_create: IBM %d bound to another solver", i);
        for (int j = 0; j < i; ++j)
            if (solvers[j] == s) return fail(CLBM_ERR_ARG, "clbm_ensemble_create: solver %d repeated", i);
    }
    clbm_ensemble* e = new clbm_ensemble();
    e->n = n;
    e->storage = solvers[0]->cfg.storage;
    e->cur = solvers[0]->cur;
    e->local = solvers[0]->local;
    e->macro_full = solvers[0]->macro_full;
    auto bail = [&](int rc) { clbm_ensemble_destroy(e); return rc; };
    for (int i = 0; i < n; ++i) {
        e->s.push_back(solvers[i]);
        e->ibm.push_back(ibms ? ibms[i] : nullptr);
        e->m.push_back(motions[i]);
        clbm_ibm* b = e->ibm.back();
        if (b) {
            e->max_marker_blocks = std::max(e->max_marker_blocks, (b->a.n + kEnsMarkerBlock - 1) / kEnsMarkerBlock);
            const long long warps = ((long long)b->a.n + kSpreadMarkersPerWarp - 1) / kSpreadMarkersPerWarp;
            e->max_spread_blocks = std::max(e->max_spread_blocks,
                                            (int)((warps * 32 + kSpreadBlock - 1) / kSpreadBlock));
        }
    }
    {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        e->flat_grid = 16 * std::max(sms, 1);   // blocks of kBoxBlock threads
    }
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (cudaStreamCreateWithPriority(&e->st, cudaStreamNonBlocking, hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&e->st2, cudaStreamNonBlocking, lo) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->ev_box, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->ev_bulk, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&e->ev_sync, cudaEventDisableTiming) != cudaSuccess ||
        cudaMalloc(&e->d_desc, sizeof(EnsDesc) * n) != cudaSuccess ||
        cudaMalloc(&e->d_tile0, sizeof(long long) * n) != cudaSuccess ||
        cudaMalloc(&e->d_off, sizeof(long long) * 2 * (n + 1)) != cudaSuccess)
        return bail(fail(CLBM_ERR_CUDA, "clbm_ensemble_create: stream/event/allocation failed"));
    for (clbm_solver* s : e->s) {   // members' queued work (initialisation) comes first
        if (join_bulk(s) != CLBM_OK ||
            cudaEventRecord(e->ev_sync, s->st) != cudaSuccess ||
            cudaStreamWaitEvent(e->st, e->ev_sync, 0) != cudaSuccess)
            return bail(fail(CLBM_ERR_CUDA, "clbm_ensemble_create: stream ordering failed"));
    }
    const char* step_env = std::getenv("CLBM_ENS_STEP");
    if (step_env && !std::strcmp(step_env, "persistent")) {
        // descriptors only: the persistent step has its own bulk tiles
        if (int rc = ens_upload(e, 128)) return bail(rc);
        if (int rc = ens_pers_setup(e)) return bail(rc);
    } else if (int rc = ens_tune(e)) {
        return bail(rc);
    }
    *out = e;
    return CLBM_OK;
}

int clbm_ensemble_run(clbm_ensemble* e, int32_t nsteps, int32_t use_graph) {
    if (!e || nsteps < 0) return fail(CLBM_ERR_ARG, "clbm_ensemble_run: invalid argument");
    for (int i = 0; i < e->n; ++i)
        if (e->s[i]->cur != e->cur || (e->ibm[i] && e->ibm[i]->s != e->s[i]))
            return fail(CLBM_ERR_STATE, "clbm_ensemble_run: member %d was stepped or destroyed "
                        "outside the ensemble", i);
    if (int rc = ens_pers_check(e, "clbm_ensemble_run")) return rc;
    for (int i = 0; i < e->n; ++i) {
        clbm_solver* s = e->s[i];
        if (int rc = join_bulk(s)) return rc;
        if (e->ibm[i])   // a member's own compute_force that no step completed
            if (int rc = flush_sums(e->ibm[i])) return rc;
        CK(cudaEventRecord(e->ev_sync, s->st));
        CK(cudaStreamWaitEvent(e->st, e->ev_sync, 0));
    }
    int done = 0;
    while (done < nsteps && (!use_graph || e->local || e->macro_full)) {
        if (int rc = ens_step(e)) return rc;
        ++done;
    }
    if (use_graph && nsteps - done >= 2) {
        if (!e->gexec || e->g_cur != e->cur) {
            ens_free_graph(e);
            const int cur0 = e->cur;
            const long long l0 = e->launches;
            CK(cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal));
            int rc = ens_step(e);
            if (!rc) rc = ens_step(e);
            cudaGraph_t g = nullptr;
            cudaError_t err = cudaStreamEndCapture(e->st, &g);
            e->cur = cur0;
            e->launches = l0;
            if (rc) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            if (err != cudaSuccess)
                return fail(CLBM_ERR_CUDA, "clbm_ensemble_run: capture failed: %s", cudaGetErrorString(err));
            err = cudaGraphInstantiateWithFlags(&e->gexec, g, cudaGraphInstantiateFlagUseNodePriority);
            cudaGraphDestroy(g);
            if (err != cudaSuccess)
                return fail(CLBM_ERR_CUDA, "clbm_ensemble_run: instantiate failed: %s", cudaGetErrorString(err));
            e->g_cur = cur0;
        }
        while (nsteps - done >= 2) {
            CK(cudaGraphLaunch(e->gexec, e->st));
            done += 2;
            e->launches += 2 * ens_step_launches(e);
        }
    }
    while (done < nsteps) {
        if (int rc = ens_step(e)) return rc;
        ++done;
    }
    // members see the new state: host mirrors, and their streams wait for the ensemble
    CK(cudaEventRecord(e->ev_sync, e->st));
    for (int i = 0; i < e->n; ++i) {
        clbm_solver* s = e->s[i];
        if (nsteps > 0) {
            s->cur = e->cur;
            s->local = false;
            s->macro_full = false;
            s->version += nsteps;
        }
        if (e->ibm[i]) e->ibm[i]->calls += nsteps;
        CK(cudaStreamWaitEvent(s->st, e->ev_sync, 0));
    }
    return CLBM_OK;
}

int clbm_ensemble_stream(const clbm_ensemble* e, void** out) {
    if (!e || !out) return fail(CLBM_ERR_ARG, "clbm_ensemble_stream: null argument");
    *out = (void*)e->st;
    return CLBM_OK;
}

int clbm_ensemble_tuning(const clbm_ensemble* e, int32_t* tile_width, int32_t* blocks,
                         int64_t* tiles, float* bulk_ms, int32_t* rows_per_block) {
    if (!e) return fail(CLBM_ERR_ARG, "clbm_ensemble_tuning: null ensemble");
    if (rows_per_block) *rows_per_block = e->rows ? e->rows_per_tile : 0;
    long long rows = 0;
    for (const auto& G : e->groups) rows += G.ntiles;
    if (e->members) {   // one launch per member
        if (tile_width) *tile_width = -1;
        if (blocks) *blocks = e->n;
        if (tiles) *tiles = e->n;
        if (bulk_ms) *bulk_ms = e->bulk_ms;
        return CLBM_OK;
    }
    if (tile_width) *tile_width = e->rows ? 0 : e->bx;
    if (blocks) *blocks = e->rows ? (int)std::min<long long>(rows, 1LL << 30) : e->grid;
    if (tiles) *tiles = e->rows ? rows : e->ntiles;
    if (bulk_ms) *bulk_ms = e->bulk_ms;
    return CLBM_OK;
}

int clbm_ensemble_schedule(const clbm_ensemble* e, int32_t* persistent, int32_t* blocks) {
    if (!e) return fail(CLBM_ERR_ARG, "clbm_ensemble_schedule: null ensemble");
    if (persistent) *persistent = e->pers ? 1 : 0;
    if (blocks) *blocks = e->pers ? e->pers_grid : 0;
    return CLBM_OK;
}

int clbm_ensemble_phase_times(clbm_ensemble* e, double* us) {
    if (!e || !us) return fail(CLBM_ERR_ARG, "clbm_ensemble_phase_times: null argument");
    if (!e->pers) return fail(CLBM_ERR_STATE, "clbm_ensemble_phase_times: not the persistent step");
    unsigned long long t[6] = {0, 0, 0, 0, 0, 0};
    CK(cudaMemcpyAsync(t, e->d_stamps, sizeof(t), cudaMemcpyDeviceToHost, e->st));
    CK(cudaStreamSynchronize(e->st));
    for (int k = 0; k < 5; ++k) us[k] = (t[k + 1] >= t[k]) ? (double)(t[k + 1] - t[k]) * 1e-3 : 0.0;
    return CLBM_OK;
}

int clbm_selftest_grid_barrier(int32_t blocks) {
    if (blocks < 1 || blocks > 16) return fail(CLBM_ERR_ARG, "clbm_selftest_grid_barrier: blocks in [1, 16]");
    unsigned* bar = nullptr;
    cudaStream_t st = nullptr;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    if (cudaMalloc(&bar, 4 * sizeof(unsigned)) != cudaSuccess) {
        cudaStreamDestroy(st);
        return fail(CLBM_ERR_CUDA, "clbm_selftest_grid_barrier: allocation failed");
    }
    unsigned h[4] = {0, 0, 0, 0};
    cudaError_t err = cudaMemsetAsync(bar, 0, sizeof(h), st);
    if (err == cudaSuccess) err = launch_ens_barrier_selftest(bar, blocks, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(h, bar, sizeof(h), cudaMemcpyDeviceToHost, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    cudaFree(bar);
    cudaStreamDestroy(st);
    if (err != cudaSuccess) return fail(CLBM_ERR_CUDA, "clbm_selftest_grid_barrier: %s", cudaGetErrorString(err));
    if (h[2])
        return fail(CLBM_ERR_STATE, "clbm_selftest_grid_barrier: bounded barrier wait gave up as "
                    "intended (bits %u, %u arrivals)", h[2], h[0]);
    return fail(CLBM_ERR_CUDA, "clbm_selftest_grid_barrier: the barrier did not report a timeout");
}

int clbm_ensemble_destroy(clbm_ensemble* e) {
    if (!e) return CLBM_OK;
    if (e->st) cudaStreamSynchronize(e->st);
    if (e->st2) cudaStreamSynchronize(e->st2);
    ens_free_graph(e);
    if (e->d_desc) cudaFree(e->d_desc);
    ens_free_groups(e);
    for (cudaStream_t st : e->gst) cudaStreamDestroy(st);
    for (cudaEvent_t ev : e->gev) cudaEventDestroy(ev);
    for (cudaStream_t st : e->mst) cudaStreamDestroy(st);
    for (cudaEvent_t ev : e->mev) cudaEventDestroy(ev);
    if (e->d_tile0) cudaFree(e->d_tile0);
    if (e->d_off) cudaFree(e->d_off);
    if (e->d_pers) cudaFree(e->d_pers);
    if (e->d_bar) cudaFree(e->d_bar);
    if (e->d_nodev) cudaFree(e->d_nodev);
    if (e->d_stamps) cudaFree(e->d_stamps);
    cudaEvent_t evs[] = {e->ev_box, e->ev_bulk, e->ev_sync};
    for (cudaEvent_t ev : evs)
        if (ev) cudaEventDestroy(ev);
    if (e->st2) cudaStreamDestroy(e->st2);
    if (e->st) cudaStreamDestroy(e->st);
    delete e;
    return CLBM_OK;
}

}  // extern "C"
