// clbm_internal.cuh -- device data layout, shared device helpers and kernel launchers.
//
// Layout in HBM (all grids): structure of arrays, x fastest, rows padded to `pitch`
// elements (a multiple of 32, so every row starts on a 128-byte boundary for float32):
//   population q of cell (x, y, z):  f[q * plane + (z * ny + y) * pitch + x]
//   scalar field of cell (x, y, z):  a[(z * ny + y) * pitch + x]
// with plane = pitch * ny * nz. The solver stores the post-collision, pre-stream state
// (f_post) and pulls from it, so one fused pass per step reads 19 and writes 19 values
// per cell. Host-visible arrays use the reference layout (x, y, z) with z fastest and are
// produced by transposing export kernels.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "../../include/clbm_gb300.h"

namespace clbm {

// D3Q19 velocity set of the reference (clbm_moving.py:21-30); the order fixes which
// populations the Zou-He inlet reconstructs.
__host__ __device__ constexpr int ex(int q) {
    return (q == 1 || q == 7 || q == 9 || q == 11 || q == 13) ? 1
         : (q == 2 || q == 8 || q == 10 || q == 12 || q == 14) ? -1 : 0;
}
__host__ __device__ constexpr int ey(int q) {
    return (q == 3 || q == 7 || q == 8 || q == 15 || q == 17) ? 1
         : (q == 4 || q == 9 || q == 10 || q == 16 || q == 18) ? -1 : 0;
}
__host__ __device__ constexpr int ez(int q) {
    return (q == 5 || q == 11 || q == 12 || q == 15 || q == 16) ? 1
         : (q == 6 || q == 13 || q == 14 || q == 17 || q == 18) ? -1 : 0;
}
// Index of the opposite direction -e_q.
__host__ __device__ constexpr int opposite(int q) {
    for (int p = 0; p < 19; ++p)
        if (ex(p) == -ex(q) && ey(p) == -ey(q) && ez(p) == -ez(q)) return p;
    return q;
}
__host__ __device__ constexpr float wq(int q) {
    return q == 0 ? 1.0f / 3.0f : (q <= 6 ? 1.0f / 18.0f : 1.0f / 36.0f);
}

struct Grid {
    int nx, ny, nz, pitch;
    long long plane;        // pitch * ny * nz
    unsigned int* status;   // device status word: non-zero after a bounded wait gave up
    int seg;                // cells per block along x of the staged stream-collide kernel
    int spin_limit;         // polls of a bounded mbarrier wait before it gives up
    int extra_tx;           // self test only: bytes a staged block expects beyond its copies
};

constexpr unsigned int kStatusWaitTimeout = 1u;
// status bit: some collision met a density below the floor or a non-finite density
constexpr unsigned int kStatusDiverged = 2u;
// status bit of the bounds-checked build: some access tested an element index outside its
// array
constexpr unsigned int kStatusBounds = 4u;

// Bounds-checked build (-DCLBM_CHECK, a separate library): the population, force-field,
// macro-field and stencil accesses of the stream-collide, band and IBM bodies test their
// element index against the array's extent first; an index outside it sets kStatusBounds
// in the solver's status word and the access is skipped (a load gives 0) instead of
// touching memory. In the normal build the test is the constant true and compiles away.
#ifdef CLBM_CHECK
constexpr bool kBoundsChecked = true;
__device__ __forceinline__ bool in_bounds(long long i, long long n, unsigned int* status) {
    if (i >= 0 && i < n) return true;
    if (status) atomicOr(status, kStatusBounds);
    return false;
}
#else
constexpr bool kBoundsChecked = false;
__device__ __forceinline__ constexpr bool in_bounds(long long, long long, unsigned int*) { return true; }
#endif

// Collision and boundary constants, rounded to float once on the host.
struct Coef {
    float one_m_sv;   // 1 - s_v
    float s_e;        // trace relaxation rate
    float ux_in, uy_in;
    float c23, c16;   // 2/3 and 1/6 of the Zou-He inlet
    float wc[19];     // w_q * (1 - s_v / 2), Guo forcing weight
    // divergence monitor: a collision whose density is below rho_floor or not finite sets
    // kStatusDiverged in *status (no monitor when status is null)
    float rho_floor;
    unsigned int* status;
};

// Learned sub-grid closure: a 19 -> 32 -> 32 -> 1 network (GELU, BF16 weights, FP32
// accumulation) maps the 19 normalised non-equilibrium central moments of a cell to one
// relaxation rate of its collision. Two forms (parameter `mode`):
//   0  higher-order rate: third- and fourth-order central moments relax with
//      s_h = 1 + span tanh(z3) (the reference fixes s_q = s_pi = 1, clbm_moving.py:186-194);
//   1  eddy viscosity: the deviatoric second-order moments relax with
//      s_eff = 1 / (1/2 + 3 nu 2^(span g)), g = tanh(z3) where positive and tanh(z3) / 20
//      below, nu the lattice viscosity: the network adds viscosity and may remove at most
//      a factor 2^(-span/20); s_v where it outputs zero.
// Parameters are one float32 array:
namespace closure {
constexpr int kIn = 19;                        // input features (moment order of M_raw)
constexpr int kHid = 32;                       // hidden width; inputs are padded to 32
constexpr int kMu = 0;                         // [19] feature means
constexpr int kSinv = 19;                      // [19] inverse feature scales
constexpr int kW1 = 40;                        // [32 out][32 in], in >= 19 zero
constexpr int kB1 = kW1 + kHid * kHid;         // [32]
constexpr int kW2 = kB1 + kHid;                // [32 out][32 in]
constexpr int kB2 = kW2 + kHid * kHid;         // [32]
constexpr int kW3 = kB2 + kHid;                // [32]
constexpr int kB3 = kW3 + kHid;                // [1]
constexpr int kSpan = kB3 + 1;                 // [1] output range
constexpr int kMode = kSpan + 1;               // [1] 0 higher-order rate, 1 eddy viscosity
constexpr int kNu = kMode + 1;                 // [1] lattice viscosity the training assumes
constexpr int kParams = kNu + 1;
constexpr int kTrainable = kSpan - kW1;        // W1 .. b3
// BF16 images of W1, W2 and W2^T in the K-major core-matrix layout of the MMAs.
constexpr int kImgElems = 3 * kHid * kHid;
constexpr int kTargets = 9;                    // third- and fourth-order moments per sample
// Sub-grid stress targets of the eddy-viscosity form: the deviatoric parts (xy, xz, yz,
// xx - yy, xx - zz) of tau = <u u> - <u><u> (box filter of the fine velocity) and of the
// strain rate of the filtered velocity.
constexpr int kSgs = 10;
constexpr int kAux = 9;                        // filtered <u> (3) and <u u> (6) per coarse cell
constexpr int kSampleFloats = kIn + kTargets + kSgs;  // floats per training sample
constexpr int kStats = 2 * kIn + 2;            // feature sums, squares, two loss scales
}  // namespace closure

// Band box of the IBM stencils: all six entries are reduced with atomicMin, maxima stored
// negated. The reset value 0x7f7f7f7f marks an empty box.
constexpr int kBoxEmpty = 0x7f7f7f7f;

struct IbmDev {
    long long step;        // number of completed compute_force calls
    long long cur;         // index of the call whose box the next fused step uses; written by
                           // the marker kernel, so a bulk pass that starts before the
                           // force-sum kernel has advanced `step` still finds the right box
    int box[2][6];         // slot (call index & 1): imin, -imax, jmin, -jmax, kmin, -kmax
    unsigned int ticket;   // last-block detection of the force-sum kernel
    unsigned int mticket;  // last-block detection of the marker kernel
    unsigned int bticket;  // last-block detection of the box pass with the force sums
    long long ksum[2];     // box pass: exact integer sums of the clipped Eulerian force
    // slot: the Band of box[slot] (i0, ilen, j0, jlen, k0, klen, 0, 0), written by the last
    // block of the marker kernel once the box is complete, so the passes that test cells
    // against the box read six integers instead of converting the box in every thread
    alignas(16) int band[2][8];
};

// Box in lattice coordinates with periodic y/z: x in [i0, i0 + ilen), y in
// (j0 + [0, jlen)) mod ny, z in (k0 + [0, klen)) mod nz.
struct Band {
    int i0, ilen, j0, jlen, k0, klen;
};

__host__ __device__ inline int pmod(int a, int m) {
    if (a >= 0 && a < m) return a;          // the usual cases need no division
    if (a < 0 && a >= -m) return a + m;
    int r = a % m;
    return r < 0 ? r + m : r;
}

__host__ __device__ inline Band band_from_box(const int* b, int nx, int ny, int nz) {
    Band r;
    if (b[0] == kBoxEmpty || b[2] == kBoxEmpty || b[4] == kBoxEmpty) {
        r.i0 = r.j0 = r.k0 = 0;
        r.ilen = r.jlen = r.klen = 0;
        return r;
    }
    long long imin = b[0], imax = -(long long)b[1];
    long long jmin = b[2], jmax = -(long long)b[3];
    long long kmin = b[4], kmax = -(long long)b[5];
    r.i0 = (int)imin;
    r.ilen = (int)(imax - imin + 1);
    long long jl = jmax - jmin + 1, kl = kmax - kmin + 1;
    if (jl >= ny) { r.j0 = 0; r.jlen = ny; } else { r.j0 = pmod((int)jmin, ny); r.jlen = (int)jl; }
    if (kl >= nz) { r.k0 = 0; r.klen = nz; } else { r.k0 = pmod((int)kmin, nz); r.klen = (int)kl; }
    if (r.ilen <= 0 || r.jlen <= 0 || r.klen <= 0) r.ilen = r.jlen = r.klen = 0;
    return r;
}

__device__ inline bool in_band(const Band& b, int x, int y, int z, int ny, int nz) {
    int oy = y - b.j0; if (oy < 0) oy += ny;
    int oz = z - b.k0; if (oz < 0) oz += nz;
    return (unsigned)(x - b.i0) < (unsigned)b.ilen && oy < b.jlen && oz < b.klen;
}

// slot < 0: the slot of the call the device record names current (dev->cur & 1), for
// launches whose call index the host does not track (one ensemble member per launch; the
// ensemble orders the next call's marker kernel after the step).
__device__ __forceinline__ Band load_band(const IbmDev* dev, int slot) {
    if (slot < 0) slot = (int)(dev->cur & 1);
    const int4 a = *reinterpret_cast<const int4*>(dev->band[slot]);
    const int2 b = *reinterpret_cast<const int2*>(dev->band[slot] + 4);
    return Band{a.x, a.y, a.z, a.w, b.x, b.y};
}

// Cell t (0 <= t < ilen * jlen * klen) of a band box, x fastest.
__device__ __forceinline__ void box_cell(const Band& b, int ny, int nz, int t, int& x, int& y,
                                         int& z) {
    const int ox = t % b.ilen;
    const int r = t / b.ilen;
    x = b.i0 + ox;
    y = b.j0 + r % b.jlen;
    if (y >= ny) y -= ny;
    z = b.k0 + r / b.jlen;
    if (z >= nz) z -= nz;
}

// Peskin 4-point regularised delta, airfoil_moving.py:27-38, same operation order.
__device__ inline float phi1d(float r) {
    float s = fabsf(r);
    float result = 0.0f;
    if (s < 1.0f) {
        float a = 1.0f + 4.0f * s - 4.0f * s * s;
        result = (3.0f - 2.0f * s + sqrtf(fmaxf(a, 0.0f))) / 8.0f;
    } else if (s < 2.0f) {
        float a = -7.0f + 12.0f * s - 4.0f * s * s;
        result = (5.0f - 2.0f * s - sqrtf(fmaxf(a, 0.0f))) / 8.0f;
    }
    return result;
}

// ---------------------------------------------------------------- population storage
template <int S> struct Pop;
// ld/st convert between the stored value and f; ld_raw/st_raw move the stored value
// itself (f for float32, the deviation f - w for the shifted forms), for the
// deviation-form collision.
template <> struct Pop<CLBM_STORE_F32> {
    using T = float;
    static constexpr bool kShifted = false;
    static __device__ __forceinline__ float ld(const T* p, int q) { (void)q; return __ldg(p); }
    static __device__ __forceinline__ void st(T* p, int q, float v) { (void)q; *p = v; }
    static __device__ __forceinline__ float ld_raw(const T* p) { return __ldg(p); }
    static __device__ __forceinline__ void st_raw(T* p, float v) { *p = v; }
};
template <> struct Pop<CLBM_STORE_F16S> {
    using T = __half;
    static constexpr bool kShifted = true;
    static __device__ __forceinline__ float ld(const T* p, int q) {
        return __half2float(__ldg(p)) + wq(q);
    }
    static __device__ __forceinline__ void st(T* p, int q, float v) {
        *reinterpret_cast<unsigned short*>(p) = __half_as_ushort(__float2half_rn(v - wq(q)));
    }
    static __device__ __forceinline__ float ld_raw(const T* p) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ void st_raw(T* p, float v) {
        *reinterpret_cast<unsigned short*>(p) = __half_as_ushort(__float2half_rn(v));
    }
};
template <> struct Pop<CLBM_STORE_BF16S> {
    using T = __nv_bfloat16;
    static constexpr bool kShifted = true;
    static __device__ __forceinline__ float ld(const T* p, int q) {
        return __bfloat162float(__ldg(p)) + wq(q);
    }
    static __device__ __forceinline__ void st(T* p, int q, float v) {
        *reinterpret_cast<unsigned short*>(p) = __bfloat16_as_ushort(__float2bfloat16_rn(v - wq(q)));
    }
    static __device__ __forceinline__ float ld_raw(const T* p) { return __bfloat162float(__ldg(p)); }
    static __device__ __forceinline__ void st_raw(T* p, float v) {
        *reinterpret_cast<unsigned short*>(p) = __bfloat16_as_ushort(__float2bfloat16_rn(v));
    }
};

inline size_t store_bytes(int storage) { return storage == CLBM_STORE_F32 ? 4 : 2; }

// ---------------------------------------------------------------- launchers
// Force source of the fused step.
// kForceSkipBand: bulk pass of an IBM step that leaves the cells of the force box to
// launch_stream_collide_box, so the bulk can run while the IBM kernels compute the forces.
// kForceOnlyBand: the complement, the box pass: only the cells of the force box, forced.
enum ForceMode { kForceNone = 0, kForceBand = 1, kForceDense = 2, kForceSkipBand = 3, kForceOnlyBand = 4 };

// IBM force fields are accumulated in 64-bit fixed point with kForceScale units per unit
// force: integer atomics are associative, so spreading is deterministic, and a float32
// contribution scaled by a power of two converts exactly whenever |v| >= 2^-17.
constexpr float kForceScale = 1099511627776.0f;         // 2^40
constexpr float kForceInvScale = 1.0f / 1099511627776.0f;

__device__ __forceinline__ float qforce(long long v) { return (float)v * kForceInvScale; }

struct ForceArgs {
    const float* fx;       // dense mode, padded layout
    const float* fy;
    const float* fz;
    const long long* qx;   // band mode: fixed-point IBM fields, padded layout
    const long long* qy;
    const IbmDev* dev;     // band mode: boxes of the compute_force calls
    int slot;              // band mode: box slot of the call this step applies (call index & 1),
                           // passed by the host so the next call's marker kernel may run
                           // while this step's bulk pass still reads it; -1: read on the
                           // device (load_band)
};

int knob(const char* name, int def);  // integer tuning parameter from the environment
bool spread_tiled();                  // IBM spreading through shared-memory tiles (CLBM_SPREAD)
void launch_init(int storage, void* f, const Grid& g, const Coef& c, cudaStream_t st);
// One index test past the end of the populations, no access (kStatusBounds in the
// bounds-checked build).
void launch_bounds_selftest(const Grid& g, cudaStream_t st);
// binaryVersion / ptxVersion of the float32 bulk stream-collide kernel (cudaFuncGetAttributes).
cudaError_t stream_collide_binary_version(int* binary, int* ptx);
// Stream-collide kernel variants for the full-grid pass:
//   kVariantCell    one cell per thread, direct loads (float32 parity kernel)
//   kVariantPair    two cells per thread, half2 loads, warp-shuffle x shifts (16-bit only)
//   kVariantStaged  two cells per thread, rows staged in shared memory by bulk TMA copies
enum Variant { kVariantCell = 0, kVariantPair = 1, kVariantStaged = 2 };
constexpr int kVariants = 3;
void launch_stream_collide(int storage, bool pull, int fmode, int variant, const void* fin,
                           void* fout, const Grid& g, const Coef& c, const ForceArgs& fa,
                           cudaStream_t st);
// Cells per block of the staged variant for a lattice width.
int staged_segment(int nx);

// z-vorticity dux/dy - duy/dx of plane z into out (Nx, Ny), NumPy gradient edge rules.
void launch_vorticity_slice(const float* ux, const float* uy, const Grid& g, int z, float* out,
                            cudaStream_t st);

// Record the message clbm_last_error() returns on this thread.
void set_last_error(const char* msg);
// Forced stream-collide of the cells of the current IBM force box, by rows of the box;
// max_bx, max_by, max_bz bound the box size (grid sizing only).
void launch_stream_collide_box(int storage, bool pull, const void* fin, void* fout,
                               const Grid& g, const Coef& c, const ForceArgs& fa, int max_bx,
                               int max_by, int max_bz, cudaStream_t st);
struct IbmArrays;
// The same box pass, also computing the force sums of the call whose box it is into the
// history ring and advancing the device call counter (ibm_box_sums_tail).
void launch_stream_collide_box_sums(int storage, bool pull, const void* fin, void* fout,
                                    const Grid& g, const Coef& c, const ForceArgs& fa,
                                    const IbmArrays& a, cudaStream_t st);
// Macro (rho, u without force) of the current state for every cell of the grid; optional
// statistics into stats[0..3] (ordered-int min rho, max rho, max |u|^2, nonfinite count).
void launch_macro_full(int storage, bool pull, const void* f, const Grid& g, const Coef& c,
                       float* rho, float* ux, float* uy, float* uz,
                       unsigned long long* stats, cudaStream_t st);
void launch_fill_macro(const Grid& g, const Coef& c, float* rho, float* ux, float* uy,
                       float* uz, cudaStream_t st);
// Padded-layout field -> reference layout (x, y, z), optional clip to +-clipv.
void launch_export_field(const float* a, float* out, const Grid& g, float clipv,
                         cudaStream_t st);
// Same for a fixed-point IBM force field.
void launch_export_qfield(const long long* a, float* out, const Grid& g, float clipv,
                          cudaStream_t st);
// Reference layout (x, y, z) -> padded layout.
void launch_import_field(const float* in, float* a, const Grid& g, cudaStream_t st);
void launch_export_populations(int storage, bool pull, const void* f, float* out,
                               const Grid& g, const Coef& c, cudaStream_t st);
void launch_import_populations(int storage, const float* in, void* f, const Grid& g,
                               cudaStream_t st);

// IBM
struct IbmArrays {
    int n;
    const float *X0, *Y0, *Z0;
    float *X, *Y, *Z, *VX, *VY, *Uk, *Vk, *FXk, *FYk;
    long long *fx, *fy;   // padded full grid, fixed point (kForceScale)
    float *ux, *uy;       // padded full grid (macro of the solver)
    const int* perm;      // marker order of the tiled spreading: the markers sorted by the
                          // Morton code of their body-frame cell (a rigid motion keeps
                          // nearby markers nearby), so a chunk of consecutive entries is a
                          // compact cluster; outputs stay at the markers' own indices
    IbmDev* dev;
    double* hist;
    double* part;         // per-block partials: force-sum kernel [kFinishBlocks][4]; box pass
                          // marker sums [kFinishBlocks][2]
    int hist_cap;
    int max_bx, max_by, max_bz;   // upper bound of the band box dimensions
};

struct MotionF { float xc, yc, theta, vx, vy, omega; };

// Marker kinematics + band box of this call. device_motion: evaluate the motion law of
// `m` on the device for t = dev->step + 1; otherwise use the float32 values `mf`.
void launch_ibm_markers(const IbmArrays& a, const Grid& g, bool device_motion,
                        const MotionF& mf, const clbm_motion& m, cudaStream_t st);
// Zero the previous call's force band and compute the macro fields on this call's band.
constexpr int kFinishBlocks = 64;    // force-sum blocks: few, so they leave the SMs to the bulk pass
constexpr int kSpreadMarkersPerWarp = 2;   // markers interpolated and spread by one warp
// The IBM kernels run beside the bulk stream-collide pass, on a stream of higher priority.
// The block scheduler starts a waiting block only on an SM where it fits, and an SM full of
// bulk blocks frees room one bulk block at a time (64 threads x 64 registers in the 16-bit
// forms, 128 x 48 in float32): a larger block waits while the smaller low-priority blocks
// keep taking the freed room, in practice until the bulk grid runs out. The marker,
// band-prepare, spreading and box-pass kernels therefore use blocks of 64 threads (the
// 16-bit box pass with at most 64 registers).
constexpr int kMarkerBlock = 64;
// The batched marker kernel runs before the ensemble's bulk pass, not beside it: larger
// blocks there (fewer block reductions, box atomics and last-block tickets per member).
constexpr int kEnsMarkerBlock = 256;
constexpr int kBoxBlock = 64;      // band-prepare and box pass of the single lattice
constexpr int kSpreadBlock = 64;
constexpr int kTiledBlock = 256;   // shared-memory tiled spreading: 8 warps per tile
constexpr int kFinishBlock = 256;
void launch_band_prepare(int storage, bool pull, const void* f, const Grid& g, const Coef& c,
                         IbmDev* dev, long long* fx, long long* fy, float* rho, float* ux, float* uy,
                         float* uz, int max_bx, int max_by, int max_bz, bool compute_macro,
                         cudaStream_t st);
void launch_ibm_interp_spread(const IbmArrays& a, const Grid& g, cudaStream_t st);
// Force sums of this call into the history ring, then advance the device call counter.
void launch_ibm_finish(const IbmArrays& a, const Grid& g, cudaStream_t st);

// ---------------------------------------------------------------- ensemble
// Descriptor of one lattice of an ensemble: the batched kernels find everything an
// instance needs here (device copy, one entry per instance).
struct EnsDesc {
    Grid g;
    Coef c;
    void* f[2];
    float *rho, *ux, *uy, *uz;
    IbmArrays a;
    clbm_motion m;
    long long tile0;   // first bulk tile of this instance in the flat tile list
    int cells;         // nx * ny * nz
    int has_ibm;
};

// One ensemble step is seven batched launches: markers (device motion), the flat offsets
// of all force boxes, band prepare, interpolation + spreading, force sums, box pass on
// `st`; the bulk pass over the flat tile list of all instances (tile width bx, `grid`
// persistent blocks) on `st2`.
void launch_ens_markers(const EnsDesc* d, int n, int blocks, cudaStream_t st);
void launch_ens_interp_spread(const EnsDesc* d, int n, int blocks, cudaStream_t st);
void launch_ens_finish(const EnsDesc* d, int n, cudaStream_t st);
void launch_ens_bulk(int storage, bool pull, int bx, const EnsDesc* d, const long long* tile0,
                     int n, long long ntiles, int parity, int grid, cudaStream_t st);
// Whole rows per block of `threads` (a multiple of 32: >= Nx / 2 in the 16-bit forms,
// <= 256; >= Nx in float32, <= 512) over a group of instances of that row width: a tile is
// rows_per_tile consecutive rows of one instance, tile0 per instance of the group. idx32:
// every instance of the group has 19 * plane < 2^32 (32-bit element indices).
void launch_ens_bulk_rows(int storage, bool pull, int threads, int rows_per_tile, bool idx32,
                          const EnsDesc* d, const long long* tile0, int n, long long ntiles,
                          int parity, int grid, cudaStream_t st);
// The whole ensemble step as one cooperative launch of `grid` blocks of 256 threads
// (ensemble.cu, kb_step_persistent). Offsets per member (n + 1 entries each): mk0 virtual
// marker blocks of 256 markers, sw0 spreading warps; off_rows (written by the launch):
// box-pass warp items of this call's boxes (16-bit forms); the bulk pass's block tiles
// [bt_split[k], bt_split[k + 1]) are done in phase k + 2; bar: arrivals, generation, error
// bits of the grid barrier (arrivals zero at launch).
struct EnsPersArgs {
    long long* off_new;
    long long* off_old;
    long long* off_rows;
    const long long* mk0;
    const long long* sw0;
    long long mk_total, sw_total;
    int bt_split[5];
    unsigned* bar;
    const IbmDev* nodev;   // zeroed: an empty force band, for members without a body
    unsigned long long* stamps;   // optional phase clock: global timer at the start, after
                                  // each barrier and at block 0's end (6 entries)
    int n;
    int parity;
    int compute_macro;
    int fin_blocks;
};
// What the bulk tiles of the persistent step read of a member, passed in the kernel's
// parameter table (the constant bank, indexed by a block-uniform member number), so the
// bulk bodies keep the grid and collision constants out of per-thread registers as the
// separate launches do. A block tile is kPersTileWarps consecutive warp tiles of one member
// (64-cell row segments in the 16-bit forms, 32-cell runs in float32); bt0: first block
// tile of each member (n + 1 entries).
constexpr int kPersMaxMembers = 128;
constexpr int kPersTileWarps = 8;
struct EnsMember {
    Grid g;
    Coef c;
    void* f[2];
    IbmDev* dev;      // the member's IBM device state, or the zeroed one (no body)
    int cells;
    int wtiles;       // warp tiles of the member
};
struct EnsPersTable {
    EnsMember m[kPersMaxMembers];
    int bt0[kPersMaxMembers + 1];
};
// Resident blocks per SM of the persistent step (0 when the query fails).
int ens_persistent_blocks_per_sm(int storage, bool idx32);
cudaError_t launch_ens_persistent(int storage, bool pull, bool idx32, const EnsDesc* d,
                                  const EnsPersArgs& p, const EnsPersTable& t, int grid,
                                  cudaStream_t st);
// Cooperative launch whose barrier waits for one block more than it has: every wait runs
// out after its bound and sets bar[2] (failure detection without a fault).
cudaError_t launch_ens_barrier_selftest(unsigned* bar, int grid, cudaStream_t st);
// Force-box cells of all members as one flat list (offsets per member, n + 1 each), then
// band-prepare and box pass over it with `grid` blocks of kBoxBlock threads.
void launch_ens_box_scan(const EnsDesc* d, int n, long long* off_new, long long* off_old, cudaStream_t st);
void launch_ens_band_prepare_flat(int storage, bool pull, const EnsDesc* d, int n, const long long* off_new,
                                  const long long* off_old, int parity, bool compute_macro, int grid,
                                  cudaStream_t st);
void launch_ens_box_flat(int storage, bool pull, const EnsDesc* d, int n, const long long* off_new, int parity,
                         int grid, cudaStream_t st);

// ---- learned closure (closure.cu)
struct ClosureArgs {
    const float* params;      // closure parameter array (closure::kParams floats)
    const uint16_t* img;      // BF16 weight images (closure::kImgElems)
    long long cells;          // nx * ny * nz
    long long tiles;          // set by the launcher from its tile size
};

struct TrainArgs {
    const float* samples;     // samples[i * stride + j]: 19 features, then 9 targets
    long long stride;
    long long off, count;     // sample range
    long long batch;          // samples per call (random: drawn from the range with a hash)
    unsigned long long seed;
    int random;
    int spin_limit;
    const float* params;
    const uint16_t* img;
    float wscale;             // loss scale
    float* part;              // per-block partials (closure_part_floats() each)
    unsigned int* status;
};

void launch_closure_images(const float* params, uint16_t* img, cudaStream_t st);
int closure_grid(int storage);
void launch_closure_stream_collide(int storage, bool pull, int fmode, const void* fin, void* fout,
                                   const Grid& g, const Coef& c, const ForceArgs& fa,
                                   const ClosureArgs& ca, int grid, cudaStream_t st);
void launch_filter2(bool pull, const float* ff, const Grid& gf, const Coef& cf, float* out,
                    const Grid& gc, cudaStream_t st);
void launch_closure_samples(const float* f0, const float* f1, const Grid& gc, const long long* cells,
                            long long n, float* samples, long long stride, long long offset,
                            cudaStream_t st);
void launch_sample_stats(const float* s, long long stride, long long n, double* part, int blocks,
                         double* out, cudaStream_t st);
int closure_train_smem();
int closure_part_floats();
void launch_closure_train(const TrainArgs& a, bool grad, int grid, cudaStream_t st);
void launch_closure_reduce(const float* part, int blocks, float inv_batch, float* grad, double* loss,
                           cudaStream_t st);
void launch_closure_adam(float* params, const float* grad, float* m1, float* m2, float lr, float b1,
                         float b2, float eps, int t, cudaStream_t st);
void launch_tc_selftest(const float* A, const float* B, float* D, int kdim, int n, unsigned int* status,
                        int spin, cudaStream_t st);

}  // namespace clbm
