// Total cost without any device-memory allocation.
//
// Some callers cannot let a library allocate GPU memory: services that give
// each component a fixed slice of the device up front and route every other
// byte through their own pool, and latency-critical threads that must not
// hit cudaFree's device-wide synchronisation or an allocator's page faults.
// For them, sfmba_total_cost_noalloc computes the same robust cost as
// sfmba_total_cost (sum of w |r|^2 over the observations in front of their
// camera) from arrays the caller already holds in device memory, and writes
// the result to a device location the caller provides.
//
// The per-block partial sums that sfmba_total_cost keeps in its workspace
// live here in one fixed array compiled into the library
// (`g_noalloc_scratch`, 32 KB + a flag). Every GPU this library is used on
// holds that array until the process exits. Its size bounds the problem:
// at most kNoAllocMaxObservations observations (4096 blocks x 4096
// observations). All calls on a device share the array and it keeps the
// previous call's contents; each call overwrites every partial it later
// reads and clears the bad-index flag before its kernels run, so stale data
// from an earlier call is never used. Two calls whose kernels overlap on the
// GPU (different streams, or different host threads on one device) race on
// the array and may both return wrong sums: serialise them.
//
// Validation matches sfmba_total_cost: every observation's image and point
// index, every image's camera index and every camera's model id are
// checked on the device before use; any bad entry makes the call return
// SFMBA_ERR_INVALID_ARGUMENT (and NaN in the output).
//
// The host needs the array's device address, which is not the address of
// the host-side symbol; the first call on each device looks it up with
// cudaGetSymbolAddress (with that device current) and caches it. Every call
// then reads the bad-index flag back into host memory and waits for its
// stream, so the call returns only once the result is in place and cannot be
// made on a stream that is being captured into a CUDA graph.
#include <mutex>

#include "camera.cuh"

namespace sfmba {

void record_error(const char *message);

namespace {

constexpr int kNoAllocThreads = 256;
constexpr long long kNoAllocObsPerBlock = 4096;
constexpr int kNoAllocMaxBlocks = 4096;
constexpr long long kNoAllocMaxObservations = kNoAllocObsPerBlock * kNoAllocMaxBlocks;
constexpr int kMaxDevices = 64;

struct NoAllocScratch {
    double sum[kNoAllocMaxBlocks];
    int bad_index;
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_noalloc_mutex;
NoAllocScratch *g_noalloc_ptr[kMaxDevices] = {};

// Per-block partial of the robust cost; indices are range-checked so a bad
// array is reported instead of read out of bounds. The blocks also check
// every image's camera index and every camera's model, as sfmba_total_cost
// does on the host, including entries no observation reaches.
__global__ void __launch_bounds__(kNoAllocThreads)
    k_cost_noalloc_partials(sfmba_problem p, int loss, double scale, NoAllocScratch *scr) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < p.num_images + p.num_cameras;
         k += stride) {
        const bool bad = k < p.num_images
                             ? (p.camera_of_image[k] < 0 || p.camera_of_image[k] >= p.num_cameras)
                             : model_dof(p.camera_model[k - p.num_images]) == 0;
        if (bad) atomicOr(&scr->bad_index, 1);
    }
    const long long begin = blockIdx.x * kNoAllocObsPerBlock;
    long long end = begin + kNoAllocObsPerBlock;
    if (end > p.num_observations) end = p.num_observations;
    double sum = 0.0;
    for (long long o = begin + threadIdx.x; o < end; o += blockDim.x) {
        const int i = p.obs_image[o], pt = p.obs_point[o];
        if (i < 0 || i >= p.num_images || pt < 0 || pt >= p.num_points) {
            atomicOr(&scr->bad_index, 1);
            continue;
        }
        const int c = p.camera_of_image[i];
        if (c < 0 || c >= p.num_cameras || model_dof(p.camera_model[c]) == 0) {
            atomicOr(&scr->bad_index, 1);
            continue;
        }
        const double *X = p.points + 3 * (size_t)pt;
        double rx, ry;
        if (residual64(p.poses + 7 * (size_t)i, p.camera_model[c], p.camera_params + 8 * (size_t)c, X[0], X[1],
                       X[2], p.obs_xy[2 * o], p.obs_xy[2 * o + 1], rx, ry)) {
            const double n = sqrt(rx * rx + ry * ry);
            sum += robust_weight<double>(n, loss, scale) * n * n;
        }
    }
    __shared__ double ssum[kNoAllocThreads];
    ssum[threadIdx.x] = sum;
    __syncthreads();
    for (int w = kNoAllocThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) ssum[threadIdx.x] += ssum[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) scr->sum[blockIdx.x] = ssum[0];
}

// Sums the partials this call wrote, in a fixed order.
__global__ void __launch_bounds__(kNoAllocThreads)
    k_cost_noalloc_finalize(const NoAllocScratch *scr, int nblocks, double *out) {
    __shared__ double ssum[kNoAllocThreads];
    double s = 0.0;
    for (int k = threadIdx.x; k < nblocks; k += blockDim.x) s += scr->sum[k];
    ssum[threadIdx.x] = s;
    __syncthreads();
    for (int w = kNoAllocThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) ssum[threadIdx.x] += ssum[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = scr->bad_index ? __longlong_as_double(0x7ff8000000000000LL) : ssum[0];
}

// Device address of the scratch array on the current device (looked up
// once per device).
int scratch_on_current_device(NoAllocScratch **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        (void)cudaGetLastError();
        record_error("sfmba_total_cost_noalloc: no usable current CUDA device");
        return SFMBA_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            (void)cudaGetLastError();
            record_error("sfmba_total_cost_noalloc: cudaGetSymbolAddress of the scratch array failed");
            return SFMBA_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = static_cast<NoAllocScratch *>(ptr);
    }
    *out = g_noalloc_ptr[dev];
    return SFMBA_OK;
}

}  // namespace

}  // namespace sfmba

using namespace sfmba;

extern "C" int sfmba_total_cost_noalloc(const sfmba_problem *p, const sfmba_options *o, double *dev_out,
                                        void *stream) {
    record_error("");
    if (!p || !dev_out) {
        record_error("sfmba_total_cost_noalloc: problem or output is NULL");
        return SFMBA_ERR_INVALID_ARGUMENT;
    }
    if (p->num_observations < 0 || p->num_images < 0 || p->num_cameras < 0 || p->num_points < 0) {
        record_error("sfmba_total_cost_noalloc: negative size");
        return SFMBA_ERR_INVALID_ARGUMENT;
    }
    if (p->num_observations > kNoAllocMaxObservations) {
        record_error("sfmba_total_cost_noalloc: more than 16777216 observations (the fixed scratch array "
                     "holds 4096 partial sums of 4096 observations); use sfmba_total_cost");
        return SFMBA_ERR_INVALID_ARGUMENT;
    }
    if (p->num_images > (1 << 20) || p->num_cameras > (1 << 20)) {
        record_error("sfmba_total_cost_noalloc: problem too large for 32-bit indices");
        return SFMBA_ERR_INVALID_ARGUMENT;
    }
    if ((p->num_observations > 0 && (!p->obs_image || !p->obs_point || !p->obs_xy || !p->points)) ||
        (p->num_images > 0 && (!p->poses || !p->camera_of_image)) ||
        (p->num_cameras > 0 && (!p->camera_model || !p->camera_params))) {
        record_error("sfmba_total_cost_noalloc: a problem array is NULL");
        return SFMBA_ERR_INVALID_ARGUMENT;
    }
    int loss = SFMBA_LOSS_HUBER;
    double scale = 2.0;
    if (o) {
        if (o->robust_loss < 0 || o->robust_loss > 2) {
            record_error("sfmba_total_cost_noalloc: unknown robust_loss");
            return SFMBA_ERR_INVALID_ARGUMENT;
        }
        loss = o->robust_loss;
        scale = o->loss_scale_px;
    }
    NoAllocScratch *scr = nullptr;
    int st = scratch_on_current_device(&scr);
    if (st != SFMBA_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nblocks = (int)((p->num_observations + kNoAllocObsPerBlock - 1) / kNoAllocObsPerBlock);
    cudaError_t e = cudaMemsetAsync(&scr->bad_index, 0, sizeof(int), s);
    if (e == cudaSuccess && (nblocks > 0 || p->num_images + p->num_cameras > 0)) {
        // at least one block, so the image and camera checks run without observations
        k_cost_noalloc_partials<<<nblocks > 0 ? nblocks : 1, kNoAllocThreads, 0, s>>>(*p, loss, scale, scr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_cost_noalloc_finalize<<<1, kNoAllocThreads, 0, s>>>(scr, nblocks, dev_out);
        e = cudaGetLastError();
    }
    int bad = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, &scr->bad_index, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        record_error(cudaGetErrorString(e));
        return SFMBA_ERR_CUDA;
    }
    if (bad) {
        record_error("sfmba_total_cost_noalloc: observation, image or camera index out of range, or an "
                     "unknown camera model id");
        return SFMBA_ERR_INVALID_ARGUMENT;
    }
    return SFMBA_OK;
}
