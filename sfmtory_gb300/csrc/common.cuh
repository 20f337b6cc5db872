// Shared definitions of the GB300 bundle adjuster (device + host).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/sfmba.h"

namespace sfmba {

// Error carried from any CUDA call or validation failure up to the C ABI.
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

#define SFMBA_CUDA(call)                                                                       \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            (void)cudaGetLastError();                                                          \
            throw ::sfmba::Error(e_ == cudaErrorMemoryAllocation ? SFMBA_ERR_OUT_OF_MEMORY     \
                                                                 : SFMBA_ERR_CUDA,             \
                                 std::string(#call) + ": " + cudaGetErrorString(e_) + " at " + \
                                     __FILE__ + ":" + std::to_string(__LINE__));               \
        }                                                                                      \
    } while (0)

// Kernel launches of this library on the calling thread (benchmark bookkeeping).
extern thread_local long long g_kernel_launches;

#define SFMBA_LAUNCH_CHECK()                \
    do {                                    \
        ++::sfmba::g_kernel_launches;       \
        SFMBA_CUDA(cudaGetLastError());     \
    } while (0)

constexpr int kMaxParams = SFMBA_MAX_CAMERA_PARAMS;
constexpr double kMinDepth = 1e-9;            // crates/sfm-ba/src/lib.rs:256, 338
constexpr double kFunctionTolerance = 1e-6;   // lib.rs:814
constexpr int kMaxDampingRetries = 8;         // lib.rs:914

__host__ __device__ constexpr int model_dof(int model) {
    // crates/sfm-core/src/camera.rs:136-163 (params().len())
    return model == 0 ? 3 : model == 1 ? 4 : model == 2 ? 4 : model == 3 ? 5 : (model == 4 || model == 5) ? 8 : 0;
}

// Camera model M (a compile-time model id, or -1 for the runtime switch)
// is specialised for a block width D when every camera of a problem has
// model M and D is that model's width: the projection and its derivatives
// then compile without the switch over models.
__host__ __device__ constexpr bool model_fits_width(int M, int D) { return M >= 0 && 6 + model_dof(M) == D; }

// D rounded up to a multiple of 4 (16-byte rows of FP32 image vectors).
__host__ __device__ constexpr int pad4(int D) { return (D + 3) & ~3; }
// Index of entry c of image i in a plane layout of nI image vectors: entries
// 4k..4k+3 of every image form plane k ([nI] float4), so a warp reading one
// plane for neighbouring images touches a few 128-byte lines, not one line
// per image.
__host__ __device__ __forceinline__ size_t plane_index(int nI, int i, int c) {
    return ((size_t)(c >> 2) * nI + i) * 4 + (c & 3);
}
// FP32 PCG: entry c of image i of the direction vector p into its plane copy
// (the point pass's gathers read p there).
__device__ __forceinline__ void store_dir(float *p4, int nI, int i, int c, float v) { p4[plane_index(nI, i, c)] = v; }

// Width of the per-image variable block: 6 pose columns + the widest camera.
__host__ __device__ constexpr int block_width_for(int kmax) {
    return kmax == 0 ? 6 : kmax <= 3 ? 9 : kmax <= 4 ? 10 : kmax <= 5 ? 11 : 14;
}

// Per-observation linearisation record, array-of-structs, padded to 16 bytes:
//   [0,2)   r~  = sqrt(w) r
//   [2,8)   Jx~ = sqrt(w) d r / d point   (2 x 3, row major)
//   [8,8+2D) Jc~ = sqrt(w) d r / d (pose | camera)  (2 x D, row major)
// Columns of fixed poses/cameras, masked camera parameters and parameters
// past the model's count are 0, so those variables drop out of every sum.
template <int D>
struct RecLayout {
    static constexpr int kJx = 2;
    static constexpr int kJc = 8;
    static constexpr int kStride = ((8 + 2 * D) + 3) / 4 * 4;
};

// Device-resident state of the Levenberg-Marquardt loop. Kernels read the
// damping from here, so captured graphs need no per-retry arguments.
struct LMState {
    double lambda;
    double nu;
    double cost;         // cost of the current (accepted) parameters
    double trial_cost;
    double cost_before;  // cost at the start of the outer iteration
    int accepted;        // last retry accepted
    int factor_failed;   // Cholesky failed in the last retry
    int solve_failed;    // LU fallback also failed
    int converged;
    long long valid_obs;
    long long trial_valid_obs;
    int pcg_iterations;  // iterations of the current solve
    int pcg_done;        // converged or broke down
    double pcg_rzbuf[2]; // r . z, double-buffered by iteration parity
    double pcg_bb;       // |b|^2 of the current solve
    double pcg_rr;       // |r|^2
    double pcg_alpha;
    double pcg_beta;
    double pcg_tol2;     // stop when |r|^2 <= tol2 |b|^2
    long long pcg_total;  // iterations summed over the whole solve
    int pcg_breakdowns;   // solves ended by p.q <= 0 or r.z <= 0 (not by the tolerance), whole solve
    int wait_timeouts;    // bounded waits of the TMA point pass that gave up (an internal error)
};

inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace sfmba
