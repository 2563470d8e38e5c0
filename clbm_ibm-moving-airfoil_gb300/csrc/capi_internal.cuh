// capi_internal.cuh -- host-side objects behind the C ABI (solver, IBM) and the error
// helpers shared by the translation units that implement entry points.
#pragma once

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <memory>
#include <vector>
#include <algorithm>

#include "clbm_internal.cuh"

namespace clbm {
namespace api {
// Record the message of a failing call for clbm_last_error() and return `code`.
int fail(int code, const char* fmt, ...);
}  // namespace api
}  // namespace clbm

#define CK(call)                                                                      \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return clbm::api::fail(CLBM_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define CK_LAUNCH()                                                                   \
    do {                                                                              \
        cudaError_t e_ = cudaGetLastError();                                          \
        if (e_ != cudaSuccess)                                                        \
            return clbm::api::fail(CLBM_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e_)); \
    } while (0)

using clbm::Grid;
using clbm::Coef;
using clbm::IbmArrays;
using clbm::kVariantStaged;

struct clbm_ibm;

struct clbm_solver {
    clbm_config cfg{};
    Grid g{};
    Coef c{};
    void* f[2] = {nullptr, nullptr};
    int cur = 0;
    bool local = true;        // f[cur] holds a post-stream state (no pull on the next read)
    bool macro_full = false;  // rho/ux/uy/uz hold the macro fields of the current state
    float *rho = nullptr, *ux = nullptr, *uy = nullptr, *uz = nullptr;
    float *dfx = nullptr, *dfy = nullptr, *dfz = nullptr;  // dense force, padded layout
    float* stage = nullptr;
    size_t stage_bytes = 0;
    unsigned long long* stats = nullptr;
    cudaStream_t st = nullptr;     // high priority: IBM chain, box pass, transfers
    cudaStream_t st2 = nullptr;    // low priority: bulk stream-collide of IBM steps
    cudaEvent_t ev_bulk = nullptr; // end of the bulk pass (joined into st)
    bool bulk_pending = false;     // the last bulk pass is not yet joined into st: the next
                                   // compute_force's marker kernel runs beside it, and every
                                   // other call joins it first
    cudaEvent_t ev_fork = nullptr; // fork point of a bulk pass without a fresh box event
    long long version = 0;         // bumped whenever f[cur] changes
    long long launches = 0;
    int variant = clbm::kVariantStaged;  // full-grid stream-collide kernel (chosen at create)
    float variant_ms[clbm::kVariants] = {};  // autotune time per launch of each variant (0: not timed)
    unsigned int* status = nullptr;
    unsigned int* h_status = nullptr;  // pinned copy of *status, written by each graph replay
    cudaEvent_t ev_replay[4] = {};     // ends of the last graph replays (divergence polling)
    // profiling of the fused kernel
    bool prof = false;
    std::vector<cudaEvent_t> ev;
    std::vector<int> ev_tag;  // per event pair: 0 bulk / plain pass, 1 box pass
    size_t ev_used = 0;
    // cached two-step graph of the time loop
    cudaGraphExec_t gexec = nullptr;
    int g_slot = -1;               // box slot parity the cached graph was captured at
    const clbm_ibm* g_ibm = nullptr;
    clbm_motion g_m{};
    int g_cur = -1;
    std::vector<clbm_ibm*> ibms;  // IBMs bound to this solver (orphaned on destroy)
    // learned closure: when set, the bulk pass of unforced and IBM steps runs the fused
    // closure kernel (parameters and BF16 weight images on the device)
    bool closure = false;
    float* cl_params = nullptr;
    uint16_t* cl_img = nullptr;
    int cl_grid = 0;
};

struct clbm_ibm {
    clbm_solver* s = nullptr;
    IbmArrays a{};
    long long calls = 0;          // host mirror of the device call counter
    cudaEvent_t ev_box = nullptr; // recorded on st after the marker kernel of compute_force
    long long box_version = -1;   // solver state version that ev_box belongs to
    // the force sums of the last compute_force are not yet in the history: the box pass of
    // the next step computes them (or, if another call needs them first, the force-sum
    // kernel does)
    mutable bool sums_pending = false;
};

