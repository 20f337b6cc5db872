// Observation filter of filter_and_reoptimize
// (crates/sfm-reconstruction/src/lib.rs:1739-1749): an observation stays if
// its point is in front of the camera (z > 1e-9) and its reprojection error
// under the given parameters is at most the threshold, with the FP64
// projection of the cost (quaternion rotation, project()). The kept
// observations are compacted in their order (CUB select on the flags).
#include <cub/cub.cuh>

#include "camera.cuh"
#include "kernels.cuh"

namespace sfmba {

namespace {

__global__ void k_filter_flags(const double *poses, const double *cams, const double *points, const int *cam_of_img,
                               const int *cam_model, const int *ob_img, const int *ob_pt, const double *ob_xy,
                               long long nO, double threshold, unsigned char *flag) {
    const long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (o >= nO) return;
    const int i = ob_img[o], p = ob_pt[o];
    const int c = cam_of_img[i];
    const double *X = points + 3 * (size_t)p;
    double rx, ry;
    const bool ok = residual64(poses + 7 * (size_t)i, cam_model[c], cams + 8 * (size_t)c, X[0], X[1], X[2],
                               ob_xy[2 * o], ob_xy[2 * o + 1], rx, ry);
    flag[o] = (ok && sqrt(rx * rx + ry * ry) <= threshold) ? 1 : 0;
}

__global__ void k_filter_gather(const int *sel, const int *count, const int *img_in, const int *pt_in,
                                const double *xy_in, const int *orig_in, int *img_out, int *pt_out, double *xy_out,
                                int *orig_out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= *count) return;
    const int o = sel[k];
    img_out[k] = img_in[o];
    pt_out[k] = pt_in[o];
    xy_out[2 * k] = xy_in[2 * (size_t)o];
    xy_out[2 * k + 1] = xy_in[2 * (size_t)o + 1];
    orig_out[k] = orig_in[o];
}

__global__ void k_filter_keep(const int *orig, long long m, unsigned char *keep) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k < m) keep[orig[k]] = 1;
}

// Per-point mean pixel reprojection error (crates/sfm-cli/src/main.rs:1076-1098):
// the point's observations are [pt_obs[p], pt_obs[p+1]) of a point-ordered
// list; those in front of their camera (z > 1e-9) are averaged, in order.
// n_out[p] = how many were.
__global__ void k_point_errors(const double *poses, const double *cams, const double *points, const int *cam_of_img,
                               const int *cam_model, const int *ob_img, const double *ob_xy, const long long *pt_obs,
                               int nP, double *err_out, int *n_out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nP) return;
    const double *X = points + 3 * (size_t)p;
    double total = 0.0;
    int n = 0;
    for (long long o = pt_obs[p]; o < pt_obs[p + 1]; ++o) {
        const int i = ob_img[o], c = cam_of_img[i];
        double rx, ry;
        if (residual64(poses + 7 * (size_t)i, cam_model[c], cams + 8 * (size_t)c, X[0], X[1], X[2], ob_xy[2 * o],
                       ob_xy[2 * o + 1], rx, ry)) {
            total += sqrt(rx * rx + ry * ry);
            ++n;
        }
    }
    err_out[p] = n > 0 ? total / n : 0.0;
    n_out[p] = n;
}

__global__ void k_filter_iota(int *v, long long n) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k < n) v[k] = (int)k;
}

}  // namespace

size_t filter_temp_bytes(long long nO) {
    size_t bytes = 0;
    SFMBA_CUDA(cub::DeviceSelect::Flagged(nullptr, bytes, (const int *)nullptr, (unsigned char *)nullptr,
                                          (int *)nullptr, (int *)nullptr, (int)(nO > 0 ? nO : 1)));
    return bytes;
}

void launch_filter_iota(int *v, long long n, cudaStream_t s) {
    if (n == 0) return;
    k_filter_iota<<<div_up(n, 256), 256, 0, s>>>(v, n);
    SFMBA_LAUNCH_CHECK();
}

void launch_filter_select(const FilterBufs &f, long long m, const double *poses, const double *cams,
                          const double *points, double threshold, cudaStream_t s) {
    if (m == 0) {
        SFMBA_CUDA(cudaMemsetAsync(f.count, 0, sizeof(int), s));
        return;
    }
    k_filter_flags<<<div_up(m, 256), 256, 0, s>>>(poses, cams, points, f.cam_of_img, f.cam_model, f.img[0], f.pt[0],
                                                   f.xy[0], m, threshold, f.flag);
    SFMBA_LAUNCH_CHECK();
    size_t bytes = f.temp_bytes;
    SFMBA_CUDA(cub::DeviceSelect::Flagged(f.temp, bytes, f.iota, f.flag, f.sel, f.count, (int)m, s));
    k_filter_gather<<<div_up(m, 256), 256, 0, s>>>(f.sel, f.count, f.img[0], f.pt[0], f.xy[0], f.orig[0], f.img[1],
                                                    f.pt[1], f.xy[1], f.orig[1]);
    SFMBA_LAUNCH_CHECK();
}

void launch_point_errors(const double *poses, const double *cams, const double *points, const int *cam_of_img,
                         const int *cam_model, const int *ob_img, const double *ob_xy, const long long *pt_obs,
                         int nP, double *err_out, int *n_out, cudaStream_t s) {
    if (nP == 0) return;
    k_point_errors<<<div_up(nP, 128), 128, 0, s>>>(poses, cams, points, cam_of_img, cam_model, ob_img, ob_xy, pt_obs,
                                                   nP, err_out, n_out);
    SFMBA_LAUNCH_CHECK();
}

void launch_filter_keep(const int *orig, long long m, unsigned char *keep, long long nO, cudaStream_t s) {
    if (nO == 0) return;
    SFMBA_CUDA(cudaMemsetAsync(keep, 0, (size_t)nO, s));
    if (m == 0) return;
    k_filter_keep<<<div_up(m, 256), 256, 0, s>>>(orig, m, keep);
    SFMBA_LAUNCH_CHECK();
}

}  // namespace sfmba
