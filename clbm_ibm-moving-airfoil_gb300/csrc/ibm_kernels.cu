// ibm_kernels.cu -- direct-forcing immersed boundary on the GPU.
//
// One compute_force call (airfoil_moving.py:230-255) is three launches, and the step that
// follows completes it:
//   k_ibm_markers        marker kinematics (airfoil_moving.py:100-127) and the box that
//                        bounds every 4x4x4 Peskin stencil of this call (block min/max,
//                        one atomicMin per block and entry); the last block writes the band
//   k_band_prepare       (lbm_kernels.cu) zero the previous call's force box
//                        (_zero_forces, airfoil_moving.py:132-137, restricted to where
//                        forces can be non-zero) and compute _macro_post velocities of the
//                        current state inside this call's box
//   k_ibm_interp_spread  two markers per warp: 64 stencil taps each, two per lane,
//                        interpolation reduced with warp shuffles (airfoil_moving.py:142-170),
//                        marker force clip (airfoil_moving.py:175-183), spreading as exact
//                        fixed-point reductions into the Eulerian fields
//                        (airfoil_moving.py:188-214)
// The step's box pass (lbm_kernels.cu, k_box_rows_*) sums the clipped Eulerian force of
// the box and the marker forces into the history ring (lift/drag) and advances the device
// call counter; k_ibm_finish does the same when the history is read, or another
// compute_force comes, before that step. The clip itself (_clip_forces,
// airfoil_moving.py:219-225) is applied where the fields are read.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "ibm_device.cuh"

namespace clbm {

template <bool DEVM>
__global__ void __launch_bounds__(kMarkerBlock) k_ibm_markers(IbmArrays a, Grid g, MotionF mf,
                                                              clbm_motion m) {
    ibm_markers_body<DEVM>(a, g, mf, m, blockIdx.x);
}

__global__ void __launch_bounds__(kSpreadBlock) k_ibm_interp_spread(IbmArrays a, Grid g) {
    const int m0 = ((blockIdx.x * kSpreadBlock + threadIdx.x) >> 5) * kSpreadMarkersPerWarp;
    if (m0 >= a.n) return;  // whole warp leaves together
    ibm_interp_spread_body<kSpreadMarkersPerWarp>(a, g, m0, threadIdx.x & 31);
}

__global__ void __launch_bounds__(kTiledBlock) k_ibm_interp_spread_tiled(IbmArrays a, Grid g) {
    ibm_interp_spread_tiled_body(a, g, blockIdx.x);
}

__global__ void __launch_bounds__(kFinishBlock) k_ibm_finish(IbmArrays a, Grid g) {
    ibm_finish_body(a, g, blockIdx.x, gridDim.x);
}

// ---------------------------------------------------------------- launchers
void launch_ibm_markers(const IbmArrays& a, const Grid& g, bool device_motion,
                        const MotionF& mf, const clbm_motion& m, cudaStream_t st) {
    const int blocks = (a.n + kMarkerBlock - 1) / kMarkerBlock;
    if (blocks == 0) return;
    if (device_motion) k_ibm_markers<true><<<blocks, kMarkerBlock, 0, st>>>(a, g, mf, m);
    else k_ibm_markers<false><<<blocks, kMarkerBlock, 0, st>>>(a, g, mf, m);
}

// Spreading form: CLBM_SPREAD=tiled accumulates blocks of consecutive markers in
// shared-memory tiles; the default spreads with one global atomic per tap (faster at the
// marker counts measured, see the design notes).
bool spread_tiled() {
    const char* e = std::getenv("CLBM_SPREAD");   // read at every launch (graphs keep theirs)
    return e && !std::strcmp(e, "tiled");
}

void launch_ibm_interp_spread(const IbmArrays& a, const Grid& g, cudaStream_t st) {
    if (spread_tiled()) {
        const int blocks = (a.n + kTileMarkers - 1) / kTileMarkers;
        if (blocks > 0) k_ibm_interp_spread_tiled<<<blocks, kTiledBlock, 0, st>>>(a, g);
        return;
    }
    const long long threads = (long long)(a.n + kSpreadMarkersPerWarp - 1) / kSpreadMarkersPerWarp * 32;
    const int blocks = (int)((threads + kSpreadBlock - 1) / kSpreadBlock);
    if (blocks == 0) return;
    k_ibm_interp_spread<<<blocks, kSpreadBlock, 0, st>>>(a, g);
}

void launch_ibm_finish(const IbmArrays& a, const Grid& g, cudaStream_t st) {
    const long long work = std::max<long long>((long long)a.max_bx * a.max_by * a.max_bz, a.n);
    int blocks = (int)std::min<long long>((work + kFinishBlock - 1) / kFinishBlock, kFinishBlocks);
    if (blocks < 1) blocks = 1;
    k_ibm_finish<<<blocks, kFinishBlock, 0, st>>>(a, g);
}

}  // namespace clbm
